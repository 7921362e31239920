/*
 * surfatt_oracle.c -- CPU oracle (test infrastructure only) for the SurfATT
 * travel-time + adjoint path.  Plain-C restatement of SurfATT 1.6.1:
 *   src/eikon_solver_2d.f90   FSM_UW_PS_cart_2d      :22-342
 *                             FSM_WENO3_PS_2d        :344-548
 *                             FSM_WENO3_PS_multi_2d  :552-761
 *                             FSM_UW_PS_lonlat_2d    :764-1126
 *                             FSM_O1_JSE_2d          :1132-1273
 *                             FSM_O1_JSE_lonlat_2d   :1276-1446
 *                             mask                   :1449-1467
 *   src/shared/utils.f90      interp2_0_dp           :917-942
 *   src/measadj.f90           run_forward/run_adjoint/run_adjoint_density :62-104
 *   src/acqui.f90 :91-161, :307-316 and src/tomo2d.f90 :145-201 (kernel sums)
 *   src/shared/parallel.f90   scatter_all_i          :1877-1903
 *
 * Parity status: unpinned by the reference (it has no tests or golden vectors
 * for this path and cannot be built here); pinned by the analytic and
 * reciprocity / finite-difference checks in the test suite.
 *
 * Fortran semantics kept on purpose (eikon_solver_2d.f90 has no
 * `implicit none`):
 *  - r1, r2, sigx, sigy, coe are implicit REAL(4): stored as float here, and
 *    products of them such as (1-r1)*(1-r2) are evaluated in float;
 *  - `min(1.0, dble)` is evaluated in double (gfortran promotes MIN arguments
 *    to the largest kind) and then rounded to the REAL(4) variable;
 *  - parameters written with default-real literals are single-rounded:
 *    pi = 3.14159265...(REAL(4)) = 3.1415927410125732, tol = 1e-4 / 1e-9 /
 *    1e-6 (REAL(4)), eps = 1e-14 (REAL(4));
 *  - loop orders (x outer, y inner), in-place Gauss-Seidel sweeps, the
 *    nint(...) loop bounds of the adjoint / WENO sweeps, and the left-to-right
 *    association of every expression.
 * Build with -ffp-contract=off so that results do not depend on the host ISA.
 */
#include "surfatt_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define IDX(ix, iy, nx) ((size_t)(ix) + (size_t)(nx) * (size_t)(iy))

/* Operation counting build (-DORC_COUNT_FLOPS): tallies, per forward visit,
 * the two-sided cases evaluated, those with Delta >= 0 and the one-sided
 * cases, and the adjoint visits, to derive the reference formulation's
 * floating-point operation count per visit. */
#ifdef ORC_COUNT_FLOPS
static long long cnt_visit, cnt_two, cnt_delta, cnt_one, cnt_adj;
#define COUNT(c) (c)++
#else
#define COUNT(c) ((void)0)
#endif

static const double PI_S = (double)3.14159265358979323846f; /* :785, :1297 */
static const double R_EARTH = 6371.0;                        /* :777, :1296 */
static const double TOL_UW = (double)1e-4f;                  /* :775 */
static const double TOL_JSE = (double)1e-9f;                 /* :1294 */
static const double TOL_WENO = (double)1e-6f;                /* :353, :559 */
static const double EPS14 = (double)1e-14f;                  /* :775, :1294 */
enum { MAXITER_UW = 2000, MAXITER_JSE = 1000, MAXITER_WENO = 1000 };

/* Fortran nint() of a REAL(4) value: round half away from zero */
static int nint_f(float v) { return (int)lroundf(v); }

/* Adjoint / WENO sweep bounds: do iix = nint(0.5+Nx/2.0+(Nx/2.0-1.5)*xdirec),
 * nint(0.5+Nx/2.0+(-Nx/2.0+1.5)*xdirec), -xdirec   (:1389-1390, :451-452).
 * Returned 0-based. */
static void sweep_bounds(int n, int direc, int* first, int* last, int* step) {
  float nh = (float)n / 2.0f;
  float fd = (float)direc;
  *first = nint_f(0.5f + nh + (nh - 1.5f) * fd) - 1;
  *last = nint_f(0.5f + nh + (-nh + 1.5f) * fd) - 1;
  *step = -direc;
}

/* Source/receiver cell and REAL(4) bilinear weights: idx0=floor((x0-xx(1))/dx+1);
 * r1 = min(1.0,(x0-xx(idx0))/dx)  (:828-829).  Returns 0-based idx0, or -1
 * when the node pair (idx0, idx0+1) would leave the grid. */
static int locate(const double* xx, int n, double dx, double x0, float* r) {
  double f = floor((x0 - xx[0]) / dx + 1.0);
  if (!(f >= 1.0) || f > (double)n) return -1;
  int i = (int)f - 1;
  double q = (x0 - xx[i]) / dx;
  *r = (float)(q < 1.0 ? q : 1.0);
  return i;
}

/* ========================================================================= */
/* First-order upwind factored sweep shared by FSM_UW_PS_cart_2d and
 * FSM_UW_PS_lonlat_2d (identical sweep bodies: :120-342 and :880-1126).     */
/* ========================================================================= */
static int uw_sweeps(int nx, int ny, double dx, double dy, const double* a, const double* b,
                     const double* c, const double* fun, const double* T0, const double* T0x,
                     const double* T0y, double* tau, const unsigned char* ischange, int* niter) {
  size_t n = (size_t)nx * ny;
  double* tau_old = (double*)malloc(n * sizeof(double));
  int status = ORC_NOT_CONVERGED, iter;
  for (iter = 1; iter <= MAXITER_UW; ++iter) {
    memcpy(tau_old, tau, n * sizeof(double));
    for (int isw = 1; isw <= 4; ++isw) {
      int xdir = (isw <= 2) ? 1 : -1;
      int ydir = (isw == 1 || isw == 3) ? 1 : -1;
      int x1 = xdir > 0 ? 0 : nx - 1, x2 = xdir > 0 ? nx : -1;
      int y1 = ydir > 0 ? 0 : ny - 1, y2 = ydir > 0 ? ny : -1;
      for (int ix = x1; ix != x2; ix += xdir) {
        for (int iy = y1; iy != y2; iy += ydir) {
          size_t k = IDX(ix, iy, nx);
          if (!ischange[k]) continue;
          COUNT(cnt_visit);
          double ak = a[k], bk = b[k], ck = c[k], fk = fun[k], t0 = T0[k];
          double t = tau[k];
          /* two-sided cases (:911-994) */
          for (int icase = 1; icase <= 4; ++icase) {
            double px, qx, py, qy;
            switch (icase) {
              case 1:
                if (ix == 0 || iy == 0) continue;
                px = (T0x[k] + t0 / dx); qx = -(t0 / dx * tau[k - 1]);
                py = (T0y[k] + t0 / dy); qy = -(t0 / dy * tau[k - nx]);
                break;
              case 2:
                if (ix == 0 || iy == ny - 1) continue;
                px = (T0x[k] + t0 / dx); qx = -(t0 / dx * tau[k - 1]);
                py = (T0y[k] - t0 / dy); qy = t0 / dy * tau[k + nx];
                break;
              case 3:
                if (ix == nx - 1 || iy == 0) continue;
                px = (T0x[k] - t0 / dx); qx = t0 / dx * tau[k + 1];
                py = (T0y[k] + t0 / dy); qy = -(t0 / dy * tau[k - nx]);
                break;
              default:
                if (ix == nx - 1 || iy == ny - 1) continue;
                px = (T0x[k] - t0 / dx); qx = t0 / dx * tau[k + 1];
                py = (T0y[k] - t0 / dy); qy = t0 / dy * tau[k + nx];
                break;
            }
            COUNT(cnt_two);
            double eqn_a = ak * (px * px) + bk * (py * py) - 2 * ck * px * py;
            double eqn_b = 2 * ak * px * qx + 2 * bk * py * qy - 2 * ck * (px * qy + py * qx);
            double eqn_c = ak * (qx * qx) + bk * (qy * qy) - 2 * ck * qx * qy - fk * fk;
            double Delta = eqn_b * eqn_b - 4 * eqn_a * eqn_c;
            if (Delta >= 0) {
              COUNT(cnt_delta);
              for (int isol = 1; isol <= 2; ++isol) {
                double tmp = (isol == 1) ? (-eqn_b + sqrt(Delta)) / (2 * eqn_a)
                                         : (-eqn_b - sqrt(Delta)) / (2 * eqn_a);
                double Tx = px * tmp + qx;
                double Ty = py * tmp + qy;
                double chx = ak * Tx - ck * Ty;
                double chy = bk * Ty - ck * Tx;
                int caus;
                switch (icase) {
                  case 1: caus = (chx >= 0 && chy >= 0); break;
                  case 2: caus = (chx >= 0 && chy <= 0); break;
                  case 3: caus = (chx <= 0 && chy >= 0); break;
                  default: caus = (chx <= 0 && chy <= 0); break;
                }
                if (caus && tmp < t) t = tmp; /* running min == min over candidates */
              }
            }
          }
          /* one-sided cases (:996-1075) */
          double disx = sqrt(fk * fk * (bk / (ak * bk - ck * ck)));
          double disy = sqrt(fk * fk * (ak / (ak * bk - ck * ck)));
          for (int icase = 1; icase <= 4; ++icase) {
            double p, q, dis;
            size_t nb;
            switch (icase) {
              case 1:
                if (ix == 0) continue;
                nb = k - 1; p = (T0x[k] + t0 / dx); q = -(t0 / dx * tau[nb]); dis = disx;
                break;
              case 2:
                if (ix == nx - 1) continue;
                nb = k + 1; p = (T0x[k] - t0 / dx); q = t0 / dx * tau[nb]; dis = disx;
                break;
              case 3:
                if (iy == 0) continue;
                nb = k - nx; p = (T0y[k] + t0 / dy); q = -(t0 / dy * tau[nb]); dis = disy;
                break;
              default:
                if (iy == ny - 1) continue;
                nb = k + nx; p = (T0y[k] - t0 / dy); q = t0 / dy * tau[nb]; dis = disy;
                break;
            }
            COUNT(cnt_one);
            double tnb = tau[nb];
            double tmp = (dis - q) / p;
            if (tmp * t0 >= tnb * T0[nb] && tmp > tnb * 0.5 && tmp < t) t = tmp;
            tmp = (-dis - q) / p;
            if (tmp * t0 >= tnb * T0[nb] && tmp > tnb * 0.5 && tmp < t) t = tmp;
          }
          tau[k] = t;
        }
      }
    }
    /* convergence (:1091-1115): x outer, y inner */
    double L1 = 0, Linf = 0;
    for (int ix = 0; ix < nx; ++ix)
      for (int iy = 0; iy < ny; ++iy) {
        size_t k = IDX(ix, iy, nx);
        double d = fabs(tau[k] - tau_old[k]) * T0[k];
        L1 = L1 + d;
        if (d > Linf) Linf = d;
      }
    L1 = L1 / (double)nx / (double)ny;
    if (fabs(L1) < TOL_UW && Linf < TOL_UW) { status = ORC_OK; break; }
  }
  if (niter) *niter = iter > MAXITER_UW ? MAXITER_UW : iter;
  free(tau_old);
  return status;
}

int orc_fsm_uw_ps_lonlat_2d(const double* xx_deg, const double* yy_deg, int nx, int ny,
                            const double* spha, const double* sphb, const double* sphc,
                            double* T, const double* fun, double x0_deg, double y0_deg,
                            int* niter) {
  if (nx < 2 || ny < 2) return ORC_BAD_ARG;
  size_t n = (size_t)nx * ny;
  double* xx = (double*)malloc(nx * sizeof(double));
  double* yy = (double*)malloc(ny * sizeof(double));
  double* w = (double*)malloc(7 * n * sizeof(double));
  unsigned char* ischange = (unsigned char*)malloc(n);
  double *a = w, *b = w + n, *c = w + 2 * n, *T0 = w + 3 * n, *T0x = w + 4 * n,
         *T0y = w + 5 * n, *tau = w + 6 * n;
  int status = ORC_OK;
  /* degrees -> radians (:801-804): xx_deg/180.0*pi */
  for (int i = 0; i < nx; ++i) xx[i] = xx_deg[i] / 180.0 * PI_S;
  for (int j = 0; j < ny; ++j) yy[j] = yy_deg[j] / 180.0 * PI_S;
  double x0 = x0_deg / 180.0 * PI_S, y0 = y0_deg / 180.0 * PI_S;
  double dx = xx[1] - xx[0], dy = yy[1] - yy[0];
  /* spherical metric (:817-821) */
  for (int j = 0; j < ny; ++j) {
    double cy = cos(yy[j]);
    for (int i = 0; i < nx; ++i) {
      size_t k = IDX(i, j, nx);
      a[k] = spha[k] / (R_EARTH * R_EARTH * (cy * cy));
      b[k] = sphb[k] / (R_EARTH * R_EARTH);
      c[k] = sphc[k] / (R_EARTH * R_EARTH * cy);
    }
  }
  /* source slowness fun0, REAL(4) weights (:828-841) */
  float r1 = 0, r2 = 0;
  int i0 = locate(xx, nx - 1, dx, x0, &r1), j0 = locate(yy, ny - 1, dy, y0, &r2);
  if (i0 < 0 || j0 < 0) { status = ORC_BAD_ARG; goto done; }
  {
    float w00 = (1 - r1) * (1 - r2), w01 = (1 - r1) * r2, w10 = r1 * (1 - r2), w11 = r1 * r2;
    double fun0 = (double)w00 * fun[IDX(i0, j0, nx)] + (double)w01 * fun[IDX(i0, j0 + 1, nx)] +
                  (double)w10 * fun[IDX(i0 + 1, j0, nx)] + (double)w11 * fun[IDX(i0 + 1, j0 + 1, nx)];
    /* T0 = great-circle distance * fun0 and its analytic gradient (:845-872) */
    for (int i = 0; i < nx; ++i) {
      for (int j = 0; j < ny; ++j) {
        size_t k = IDX(i, j, nx);
        double tmp = sin(yy[j]) * sin(y0) + cos(yy[j]) * cos(y0) * cos(xx[i] - x0);
        double cl = tmp < 1.0 ? tmp : 1.0;
        cl = cl > -1.0 ? cl : -1.0;
        T0[k] = acos(cl) * R_EARTH * fun0;
        if (T0[k] == 0) {
          T0x[k] = 0;
          T0y[k] = 0;
        } else {
          T0x[k] = -(1.0 / sqrt(1 - tmp * tmp) * cos(yy[j]) * cos(y0) * (-1.0) * sin(xx[i] - x0) *
                     R_EARTH * fun0);
          T0y[k] = -(1.0 / sqrt(1 - tmp * tmp) *
                     (cos(yy[j]) * sin(y0) - sin(yy[j]) * cos(y0) * cos(xx[i] - x0)) * R_EARTH * fun0);
        }
        if (fabs((xx[i] - x0) / dx) <= 1 && fabs((yy[j] - y0) / dy) <= 1) {
          tau[k] = 1;
          ischange[k] = 0;
          if (i == 0 || i == nx - 1 || j == 0 || j == ny - 1) { status = ORC_SOURCE_ON_BOUNDARY; goto done; }
        } else {
          tau[k] = 10;
          ischange[k] = 1;
        }
      }
    }
  }
  status = uw_sweeps(nx, ny, dx, dy, a, b, c, fun, T0, T0x, T0y, tau, ischange, niter);
  for (size_t k = 0; k < n; ++k) T[k] = tau[k] * T0[k];
done:
  free(xx); free(yy); free(w); free(ischange);
  return status;
}

/* Shared Cartesian T0 of the cart / WENO3 solvers (:47-73, :363-386, :570-593).
 * frozen_radius 1 (UW) or 2 (WENO3); tau_frozen / tau_init per variant. */
static int cart_setup(const double* xx, const double* yy, int nx, int ny, const double* a,
                      const double* b, const double* c, const double* fun, double x0, double y0,
                      double frozen_radius, double tau_frozen, double tau_init, double* T0,
                      double* T0x, double* T0y, double* tau, unsigned char* ischange) {
  double dx = xx[1] - xx[0], dy = yy[1] - yy[0];
  float r1 = 0, r2 = 0;
  int i0 = locate(xx, nx - 1, dx, x0, &r1), j0 = locate(yy, ny - 1, dy, y0, &r2);
  if (i0 < 0 || j0 < 0) return ORC_BAD_ARG;
  float w00 = (1 - r1) * (1 - r2), w01 = (1 - r1) * r2, w10 = r1 * (1 - r2), w11 = r1 * r2;
  size_t k00 = IDX(i0, j0, nx), k01 = IDX(i0, j0 + 1, nx), k10 = IDX(i0 + 1, j0, nx),
         k11 = IDX(i0 + 1, j0 + 1, nx);
  double a0 = (double)w00 * a[k00] + (double)w01 * a[k01] + (double)w10 * a[k10] + (double)w11 * a[k11];
  double b0 = (double)w00 * b[k00] + (double)w01 * b[k01] + (double)w10 * b[k10] + (double)w11 * b[k11];
  double c0 = (double)w00 * c[k00] + (double)w01 * c[k01] + (double)w10 * c[k10] + (double)w11 * c[k11];
  double fun0 = (double)w00 * fun[k00] + (double)w01 * fun[k01] + (double)w10 * fun[k10] +
                (double)w11 * fun[k11];
  double D = a0 * b0 - c0 * c0;
  for (int i = 0; i < nx; ++i) {
    for (int j = 0; j < ny; ++j) {
      size_t k = IDX(i, j, nx);
      double ddx = xx[i] - x0, ddy = yy[j] - y0;
      T0[k] = fun0 * sqrt((b0 / D * (ddx * ddx) + a0 / D * (ddy * ddy) + 2 * c0 / D * ddx * ddy));
      if (T0[k] == 0) {
        T0x[k] = 0;
        T0y[k] = 0;
      } else {
        T0x[k] = fun0 * fun0 * (b0 / D * ddx + c0 / D * ddy) / T0[k];
        T0y[k] = fun0 * fun0 * (a0 / D * ddy + c0 / D * ddx) / T0[k];
      }
      if (fabs(ddx / dx) <= frozen_radius && fabs(ddy / dy) <= frozen_radius) {
        tau[k] = tau_frozen;
        ischange[k] = 0;
        if (i == 0 || i == nx - 1 || j == 0 || j == ny - 1) return ORC_SOURCE_ON_BOUNDARY;
      } else {
        tau[k] = tau_init;
        ischange[k] = 1;
      }
    }
  }
  return ORC_OK;
}

int orc_fsm_uw_ps_cart_2d(const double* xx, const double* yy, int nx, int ny,
                          const double* a, const double* b, const double* c,
                          double* T, const double* fun, double x0, double y0, int* niter) {
  if (nx < 2 || ny < 2) return ORC_BAD_ARG;
  size_t n = (size_t)nx * ny;
  double* w = (double*)malloc(4 * n * sizeof(double));
  unsigned char* ischange = (unsigned char*)malloc(n);
  double *T0 = w, *T0x = w + n, *T0y = w + 2 * n, *tau = w + 3 * n;
  int status = cart_setup(xx, yy, nx, ny, a, b, c, fun, x0, y0, 1.0, 1.0, 10.0, T0, T0x, T0y,
                          tau, ischange);
  if (status == ORC_OK) {
    status = uw_sweeps(nx, ny, xx[1] - xx[0], yy[1] - yy[0], a, b, c, fun, T0, T0x, T0y, tau,
                       ischange, niter);
    for (size_t k = 0; k < n; ++k) T[k] = tau[k] * T0[k];
  }
  free(w); free(ischange);
  return status;
}

/* ========================================================================= */
/* WENO3 Lax-Friedrichs sweeps (:344-548 additive, :552-761 multiplicative)   */
/* ========================================================================= */
/* WENO weight 1.0/(1+2*((eps+(u)**2)/(eps+(v)**2))**2) */
static double weno_w(double u, double v) {
  double r = (EPS14 + u * u) / (EPS14 + v * v);
  return 1.0 / (1 + 2 * (r * r));
}

/* one-direction WENO3 derivative pair (p1, p2) at index i along a line with
 * stride s (x: 1, y: nx); branch on i == 1 / i == n-2 as the reference does */
static void weno_pair(const double* tau, size_t k, size_t s, int i, int n, double h, double* p1,
                      double* p2) {
  double tm2 = 0, tm1 = tau[k - s], t0 = tau[k], tp1 = tau[k + s], tp2 = 0;
  if (i == 1) {
    tp2 = tau[k + 2 * s];
    *p1 = (t0 - tm1) / h;
    double w2 = weno_w(t0 - 2 * tp1 + tp2, tm1 - 2 * t0 + tp1);
    *p2 = (1 - w2) * (tp1 - tm1) / 2 / h + w2 * (-3 * t0 + 4 * tp1 - tp2) / 2 / h;
  } else if (i == n - 2) {
    tm2 = tau[k - 2 * s];
    double w1 = weno_w(t0 - 2 * tm1 + tm2, tp1 - 2 * t0 + tm1);
    *p1 = (1 - w1) * (tp1 - tm1) / 2 / h + w1 * (3 * t0 - 4 * tm1 + tm2) / 2 / h;
    *p2 = (tp1 - t0) / h;
  } else {
    tm2 = tau[k - 2 * s];
    tp2 = tau[k + 2 * s];
    double w1 = weno_w(t0 - 2 * tm1 + tm2, tp1 - 2 * t0 + tm1);
    *p1 = (1.0 - w1) * (tp1 - tm1) / 2 / h + w1 * (3 * t0 - 4 * tm1 + tm2) / 2 / h;
    double w2 = weno_w(t0 - 2 * tp1 + tp2, tm1 - 2 * t0 + tp1);
    *p2 = (1.0 - w2) * (tp1 - tm1) / 2 / h + w2 * (-3 * t0 + 4 * tp1 - tp2) / 2 / h;
  }
}

static int weno_solve(const double* xx, const double* yy, int nx, int ny, const double* a,
                      const double* b, const double* c, double* T, const double* fun, double x0,
                      double y0, int* niter, int multiplicative) {
  if (nx < 4 || ny < 4) return ORC_BAD_ARG;
  size_t n = (size_t)nx * ny;
  double* w = (double*)malloc(5 * n * sizeof(double));
  unsigned char* ischange = (unsigned char*)malloc(n);
  double *T0 = w, *T0x = w + n, *T0y = w + 2 * n, *tau = w + 3 * n, *tau_old = w + 4 * n;
  double dx = xx[1] - xx[0], dy = yy[1] - yy[0];
  int status = cart_setup(xx, yy, nx, ny, a, b, c, fun, x0, y0, 2.0,
                          multiplicative ? 1.0 : 0.0, multiplicative ? 1.0 : 20.0, T0, T0x, T0y,
                          tau, ischange);
  int iter = 0;
  if (status != ORC_OK) goto done;
  status = ORC_NOT_CONVERGED;
  for (iter = 1; iter <= MAXITER_WENO; ++iter) {
    memcpy(tau_old, tau, n * sizeof(double));
    for (int xdirec = -1; xdirec <= 1; xdirec += 2) {
      for (int ydirec = -1; ydirec <= 1; ydirec += 2) {
        int xf, xl, xs, yf, yl, ys;
        sweep_bounds(nx, xdirec, &xf, &xl, &xs);
        sweep_bounds(ny, ydirec, &yf, &yl, &ys);
        for (int ix = xf; ix != xl + xs; ix += xs) {
          for (int iy = yf; iy != yl + ys; iy += ys) {
            size_t k = IDX(ix, iy, nx);
            if (!ischange[k]) continue;
            float sigx, sigy, coe;
            if (multiplicative) {
              sigx = (float)(sqrt(a[k]) * T0[k]);
              sigy = (float)(sqrt(b[k]) * T0[k]);
            } else {
              sigx = (float)sqrt(a[k]);
              sigy = (float)sqrt(b[k]);
            }
            coe = (float)(1.0 / (((double)sigx / dx) + ((double)sigy / dy)));
            double px1, px2, py1, py2;
            weno_pair(tau, k, 1, ix, nx, dx, &px1, &px2);
            weno_pair(tau, k, (size_t)nx, iy, ny, dy, &py1, &py2);
            double Htau;
            if (multiplicative) {
              double U = T0x[k] * tau[k] + T0[k] * (px1 + px2) / 2;
              double V = T0y[k] * tau[k] + T0[k] * (py1 + py2) / 2;
              Htau = sqrt(a[k] * (U * U) + b[k] * (V * V) - 2 * c[k] * U * V);
            } else {
              double P = (px1 + px2) / 2, Q = (py1 + py2) / 2;
              Htau = sqrt(a[k] * (P * P) + b[k] * (Q * Q) - 2 * c[k] * (px1 + px2) * (py1 + py2) / 4 +
                          2 * (a[k] * T0x[k] - c[k] * T0y[k]) * (px1 + px2) / 2 +
                          2 * (b[k] * T0y[k] - c[k] * T0x[k]) * (py1 + py2) / 2 +
                          a[k] * (T0x[k] * T0x[k]) + b[k] * (T0y[k] * T0y[k]) -
                          2 * c[k] * T0x[k] * T0y[k]);
            }
            double tpT = (double)coe * (fun[k] - Htau) +
                         (double)coe * ((double)sigx * (px2 - px1) / 2 + (double)sigy * (py2 - py1) / 2) +
                         tau[k];
            tau[k] = tpT;
          }
        }
        /* boundary extrapolation after every sweep (:502-509, :715-722) */
        int jlo = multiplicative ? 1 : 0, jhi = multiplicative ? ny - 1 : ny;
        for (int iy = jlo; iy < jhi; ++iy) {
          double v1 = 2 * tau[IDX(1, iy, nx)] - tau[IDX(2, iy, nx)], v2 = tau[IDX(2, iy, nx)];
          tau[IDX(0, iy, nx)] = v1 > v2 ? v1 : v2;
          v1 = 2 * tau[IDX(nx - 2, iy, nx)] - tau[IDX(nx - 3, iy, nx)];
          v2 = tau[IDX(nx - 3, iy, nx)];
          tau[IDX(nx - 1, iy, nx)] = v1 > v2 ? v1 : v2;
        }
        int ilo = multiplicative ? 1 : 0, ihi = multiplicative ? nx - 1 : nx;
        for (int ix = ilo; ix < ihi; ++ix) {
          double v1 = 2 * tau[IDX(ix, 1, nx)] - tau[IDX(ix, 2, nx)], v2 = tau[IDX(ix, 2, nx)];
          tau[IDX(ix, 0, nx)] = v1 > v2 ? v1 : v2;
          v1 = 2 * tau[IDX(ix, ny - 2, nx)] - tau[IDX(ix, ny - 3, nx)];
          v2 = tau[IDX(ix, ny - 3, nx)];
          tau[IDX(ix, ny - 1, nx)] = v1 > v2 ? v1 : v2;
        }
      }
    }
    double L1 = 0, Linf = 0;
    for (int ix = 0; ix < nx; ++ix)
      for (int iy = 0; iy < ny; ++iy) {
        size_t k = IDX(ix, iy, nx);
        double d = fabs(tau[k] - tau_old[k]);
        L1 = L1 + d * dx * dy;
        if (d > Linf) Linf = d;
      }
    if (fabs(L1) < TOL_WENO && Linf < TOL_WENO) { status = ORC_OK; break; }
  }
  if (iter > MAXITER_WENO) iter = MAXITER_WENO;
  for (size_t k = 0; k < n; ++k) T[k] = multiplicative ? tau[k] * T0[k] : tau[k] + T0[k];
done:
  if (niter) *niter = iter;
  free(w); free(ischange);
  return status;
}

int orc_fsm_weno3_ps_multi_2d(const double* xx, const double* yy, int nx, int ny,
                              const double* a, const double* b, const double* c,
                              double* T, const double* fun, double x0, double y0, int* niter) {
  return weno_solve(xx, yy, nx, ny, a, b, c, T, fun, x0, y0, niter, 1);
}

int orc_fsm_weno3_ps_2d(const double* xx, const double* yy, int nx, int ny,
                        const double* a, const double* b, const double* c,
                        double* T, const double* fun, double x0, double y0, int* niter) {
  return weno_solve(xx, yy, nx, ny, a, b, c, T, fun, x0, y0, niter, 0);
}

/* ========================================================================= */
/* First-order adjoint sweeps (:1132-1273 Cartesian, :1276-1446 lon/lat)      */
/* ========================================================================= */
static int jse_core(const double* xx, const double* yy, int nx, int ny, const double* a,
                    const double* b, const double* c, const double* T, double* Ta,
                    const double* delta, int* niter) {
  size_t n = (size_t)nx * ny;
  double* w = (double*)malloc(9 * n * sizeof(double));
  double *a1m = w, *a1p = w + n, *a2m = w + 2 * n, *a2p = w + 3 * n, *b1m = w + 4 * n,
         *b1p = w + 5 * n, *b2m = w + 6 * n, *b2p = w + 7 * n, *OldTa = w + 8 * n;
  double dx = xx[1] - xx[0], dy = yy[1] - yy[0];
  int status = ORC_NOT_CONVERGED, iter;
  /* face coefficients (:1348-1370) */
  for (int i = 1; i < nx - 1; ++i) {
    for (int j = 1; j < ny - 1; ++j) {
      size_t k = IDX(i, j, nx);
      size_t W = k - 1, E = k + 1, S = k - nx, N = k + nx;
      double a1 = -((T[k] - T[W]) / dx * (a[k] + a[W]) / 2) +
                  (T[N] - T[S] + T[W + nx] - T[W - nx]) / (4 * dy) * (c[k] + c[W]) / 2;
      a1m[k] = (a1 - fabs(a1)) / 2; a1p[k] = (a1 + fabs(a1)) / 2;
      double a2 = -((T[E] - T[k]) / dx * (a[E] + a[k]) / 2) +
                  (T[E + nx] - T[E - nx] + T[N] - T[S]) / (4 * dy) * (c[E] + c[k]) / 2;
      a2m[k] = (a2 - fabs(a2)) / 2; a2p[k] = (a2 + fabs(a2)) / 2;
      double b1 = -((T[k] - T[S]) / dy * (b[k] + b[S]) / 2) +
                  (T[E] - T[W] + T[S + 1] - T[S - 1]) / (4 * dx) * (c[k] + c[S]) / 2;
      b1m[k] = (b1 - fabs(b1)) / 2; b1p[k] = (b1 + fabs(b1)) / 2;
      double b2 = -((T[N] - T[k]) / dy * (b[N] + b[k]) / 2) +
                  (T[N + 1] - T[N - 1] + T[E] - T[W]) / (4 * dx) * (c[N] + c[k]) / 2;
      b2m[k] = (b2 - fabs(b2)) / 2; b2p[k] = (b2 + fabs(b2)) / 2;
      Ta[k] = 100;
    }
  }
  for (int i = 0; i < nx; ++i) { Ta[IDX(i, 0, nx)] = 0; Ta[IDX(i, ny - 1, nx)] = 0; }
  for (int j = 0; j < ny; ++j) { Ta[IDX(0, j, nx)] = 0; Ta[IDX(nx - 1, j, nx)] = 0; }

  for (iter = 1; iter <= MAXITER_JSE; ++iter) {
    memcpy(OldTa, Ta, n * sizeof(double));
    for (int xdirec = -1; xdirec <= 1; xdirec += 2) {
      for (int ydirec = -1; ydirec <= 1; ydirec += 2) {
        int xf, xl, xs, yf, yl, ys;
        sweep_bounds(nx, xdirec, &xf, &xl, &xs);
        sweep_bounds(ny, ydirec, &yf, &yl, &ys);
        for (int ix = xf; ix != xl + xs; ix += xs) {
          for (int iy = yf; iy != yl + ys; iy += ys) {
            size_t k = IDX(ix, iy, nx);
            COUNT(cnt_adj);
            double d = (a2p[k] - a1m[k]) / dx + (b2p[k] - b1m[k]) / dy;
            if (fabs(d) < EPS14) {
              Ta[k] = 0;
            } else {
              double e = (Ta[k - 1] * a1p[k] - Ta[k + 1] * a2m[k]) / dx +
                         (Ta[k - nx] * b1p[k] - Ta[k + nx] * b2m[k]) / dy;
              Ta[k] = (delta[k] + e) / d;
            }
          }
        }
      }
    }
    double L1 = 0, Linf = 0;
    for (int ix = 0; ix < nx; ++ix)
      for (int iy = 0; iy < ny; ++iy) {
        size_t k = IDX(ix, iy, nx);
        double dd = fabs(Ta[k] - OldTa[k]);
        L1 = L1 + dd;
        if (dd > Linf) Linf = dd;
      }
    L1 = L1 / (double)(nx * ny);
    if (fabs(L1) < TOL_JSE && Linf < TOL_JSE) { status = ORC_OK; break; }
  }
  if (niter) *niter = iter > MAXITER_JSE ? MAXITER_JSE : iter;
  free(w);
  return status;
}

/* bilinear splat of one adjoint source; node pairs that leave the grid carry
 * zero weight for on-grid receivers and are skipped */
static void splat(double* delta, int nx, int ny, int i0, int j0, double v00, double v01,
                  double v10, double v11) {
  delta[IDX(i0, j0, nx)] += v00;
  if (j0 + 1 < ny) delta[IDX(i0, j0 + 1, nx)] += v01;
  if (i0 + 1 < nx) delta[IDX(i0 + 1, j0, nx)] += v10;
  if (i0 + 1 < nx && j0 + 1 < ny) delta[IDX(i0 + 1, j0 + 1, nx)] += v11;
}

int orc_fsm_o1_jse_lonlat_2d(const double* xx_deg, const double* yy_deg, int nx, int ny,
                             const double* spha, const double* sphb, const double* sphc,
                             const double* T, double* Ta, const double* xrec_deg,
                             const double* yrec_deg, const double* sourceAdj, int nr,
                             int* niter) {
  if (nx < 3 || ny < 3) return ORC_BAD_ARG;
  size_t n = (size_t)nx * ny;
  double* xx = (double*)malloc(nx * sizeof(double));
  double* yy = (double*)malloc(ny * sizeof(double));
  double* w = (double*)malloc(4 * n * sizeof(double));
  double *a = w, *b = w + n, *c = w + 2 * n, *delta = w + 3 * n;
  int status = ORC_OK;
  for (int i = 0; i < nx; ++i) xx[i] = xx_deg[i] / 180.0 * PI_S;
  for (int j = 0; j < ny; ++j) yy[j] = yy_deg[j] / 180.0 * PI_S;
  double dx = xx[1] - xx[0], dy = yy[1] - yy[0];
  memset(delta, 0, n * sizeof(double));
  /* delta source (:1328-1336) */
  for (int ir = 0; ir < nr; ++ir) {
    double xr = xrec_deg[ir] / 180.0 * PI_S, yr = yrec_deg[ir] / 180.0 * PI_S;
    float r1 = 0, r2 = 0;
    int i0 = locate(xx, nx, dx, xr, &r1), j0 = locate(yy, ny, dy, yr, &r2);
    if (i0 < 0 || j0 < 0) { status = ORC_BAD_ARG; goto done; }
    double den = dx * R_EARTH * cos(yr) * dy * R_EARTH;
    double s = sourceAdj[ir];
    splat(delta, nx, ny, i0, j0, s * (double)(1 - r1) * (double)(1 - r2) / den,
          s * (double)(1 - r1) * (double)r2 / den, s * (double)r1 * (double)(1 - r2) / den,
          s * (double)r1 * (double)r2 / den);
  }
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j) {
      size_t k = IDX(i, j, nx);
      double cy = cos(yy[j]);
      a[k] = spha[k] / (R_EARTH * R_EARTH * (cy * cy));
      b[k] = sphb[k] / (R_EARTH * R_EARTH);
      c[k] = sphc[k] / (R_EARTH * R_EARTH * cy);
    }
  status = jse_core(xx, yy, nx, ny, a, b, c, T, Ta, delta, niter);
done:
  free(xx); free(yy); free(w);
  return status;
}

int orc_fsm_o1_jse_2d(const double* xx, const double* yy, int nx, int ny,
                      const double* a, const double* b, const double* c,
                      const double* T, double* Ta, const double* xrec,
                      const double* yrec, const double* sourceAdj, int nr, int* niter) {
  if (nx < 3 || ny < 3) return ORC_BAD_ARG;
  size_t n = (size_t)nx * ny;
  double* delta = (double*)calloc(n, sizeof(double));
  double dx = xx[1] - xx[0], dy = yy[1] - yy[0];
  int status = ORC_OK;
  for (int ir = 0; ir < nr; ++ir) {
    float r1 = 0, r2 = 0;
    int i0 = locate(xx, nx, dx, xrec[ir], &r1), j0 = locate(yy, ny, dy, yrec[ir], &r2);
    if (i0 < 0 || j0 < 0) { status = ORC_BAD_ARG; goto done; }
    double s = sourceAdj[ir];
    splat(delta, nx, ny, i0, j0, s * (double)(1 - r1) * (double)(1 - r2) / (dx * dy),
          s * (double)(1 - r1) * (double)r2 / (dx * dy), s * (double)r1 * (double)(1 - r2) / (dx * dy),
          s * (double)r1 * (double)r2 / (dx * dy));
  }
  status = jse_core(xx, yy, nx, ny, a, b, c, T, Ta, delta, niter);
done:
  free(delta);
  return status;
}

void orc_mask(const double* xx, const double* yy, int nx, int ny, double* TableAdj, double x0,
              double y0) {
  double dx = xx[1] - xx[0], dy = yy[1] - yy[0];
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j)
      if (fabs(xx[i] - x0) < 1.5 * dx && fabs(yy[j] - y0) < 1.5 * dy) TableAdj[IDX(i, j, nx)] = 0;
}

/* interp2_0_dp: x1 = minloc(xq-x, mask=xq>=x), x2 = maxloc(xq-x, mask=xq<x) */
static int bracket(const double* x, int n, double xq, int* i1, int* i2) {
  int b1 = -1, b2 = -1;
  for (int k = 0; k < n; ++k) {
    double d = xq - x[k];
    if (xq >= x[k]) {
      if (b1 < 0 || d < xq - x[b1]) b1 = k;
    } else {
      if (b2 < 0 || d > xq - x[b2]) b2 = k;
    }
  }
  if (b1 < 0 || b2 < 0) return ORC_BAD_ARG;
  *i1 = b1;
  *i2 = b2;
  return ORC_OK;
}

int orc_interp2(const double* x, int nx, const double* y, int ny, const double* v, double xq,
                double yq, double* vq) {
  int x1, x2, y1, y2;
  if (bracket(x, nx, xq, &x1, &x2) || bracket(y, ny, yq, &y1, &y2)) return ORC_BAD_ARG;
  double vn = fabs((x[x2] - x[x1]) * (y[y2] - y[y1]));
  double N1 = fabs((x[x2] - xq) * (y[y2] - yq));
  double N2 = fabs((x[x1] - xq) * (y[y2] - yq));
  double N3 = fabs((x[x2] - xq) * (y[y1] - yq));
  double N4 = fabs((x[x1] - xq) * (y[y1] - yq));
  double r = 0;
  r = r + v[IDX(x1, y1, nx)] * (N1 / vn);
  r = r + v[IDX(x2, y1, nx)] * (N2 / vn);
  r = r + v[IDX(x1, y2, nx)] * (N3 / vn);
  r = r + v[IDX(x2, y2, nx)] * (N4 / vn);
  *vq = r;
  return ORC_OK;
}

/* ========================================================================= */
/* measadj (src/measadj.f90:62-104)                                          */
/* ========================================================================= */
int orc_run_forward(const double* xgrids, const double* ygrids, int nx, int ny,
                    const double* vel2d, const double* m11, const double* m22,
                    const double* m12, double srcx, double srcy, int nrec,
                    const double* recx, const double* recy, const double* tt,
                    const double* weight, double* timetable, double* tekio, double* chi,
                    int* niter) {
  size_t n = (size_t)nx * ny;
  double* w = (double*)malloc(2 * n * sizeof(double));
  double *vtmp = w, *nm12 = w + n;
  for (size_t k = 0; k < n; ++k) { vtmp[k] = 1.0 / vel2d[k]; nm12[k] = -m12[k]; }
  int st = orc_fsm_uw_ps_lonlat_2d(xgrids, ygrids, nx, ny, m11, m22, nm12, timetable, vtmp, srcx,
                                   srcy, niter);
  free(w);
  if (st != ORC_OK && st != ORC_NOT_CONVERGED) return st;
  double s = 0;
  for (int i = 0; i < nrec; ++i) {
    int e = orc_interp2(xgrids, nx, ygrids, ny, timetable, recx[i], recy[i], &tekio[i]);
    if (e) return e;
  }
  for (int i = 0; i < nrec; ++i) {
    double d = tekio[i] - tt[i];
    s = s + weight[i] * (d * d);
  }
  *chi = 0.5 * s;
  return st;
}

int orc_run_adjoint(const double* xgrids, const double* ygrids, int nx, int ny,
                    const double* m11, const double* m22, const double* m12,
                    double srcx, double srcy, int nrec, const double* recx,
                    const double* recy, const double* tt, const double* tekio,
                    double* weight, const double* timetable, double* adjtable, int* niter) {
  size_t n = (size_t)nx * ny;
  double* nm12 = (double*)malloc(n * sizeof(double));
  double* sadj = (double*)malloc((nrec > 0 ? nrec : 1) * sizeof(double));
  for (size_t k = 0; k < n; ++k) nm12[k] = -m12[k];
  for (int i = 0; i < nrec; ++i)
    if (fabs(tekio[i] - tt[i]) / tt[i] > 0.5) weight[i] = 0.;
  for (int i = 0; i < nrec; ++i) sadj[i] = weight[i] * (tekio[i] - tt[i]);
  int st = orc_fsm_o1_jse_lonlat_2d(xgrids, ygrids, nx, ny, m11, m22, nm12, timetable, adjtable,
                                    recx, recy, sadj, nrec, niter);
  orc_mask(xgrids, ygrids, nx, ny, adjtable, srcx, srcy);
  free(nm12); free(sadj);
  return st;
}

int orc_run_adjoint_density(const double* xgrids, const double* ygrids, int nx, int ny,
                            const double* m11, const double* m22, const double* m12,
                            double srcx, double srcy, int nrec, const double* recx,
                            const double* recy, const double* weight,
                            const double* timetable, double* density, int* niter) {
  size_t n = (size_t)nx * ny;
  double* nm12 = (double*)malloc(n * sizeof(double));
  double* sadj = (double*)malloc((nrec > 0 ? nrec : 1) * sizeof(double));
  for (size_t k = 0; k < n; ++k) nm12[k] = -m12[k];
  for (int i = 0; i < nrec; ++i) sadj[i] = -1.0 * weight[i];
  int st = orc_fsm_o1_jse_lonlat_2d(xgrids, ygrids, nx, ny, m11, m22, nm12, timetable, density,
                                    recx, recy, sadj, nrec, niter);
  orc_mask(xgrids, ygrids, nx, ny, density, srcx, srcy);
  free(nm12); free(sadj);
  return st;
}

/* ========================================================================= */
/* gradient evaluation: the per-(source, period) loop + kernel accumulation   */
/* ========================================================================= */
void orc_scatter_all_i(int countval, int size, int rank, int* istart, int* iend) {
  if (countval < size) {
    if (rank < countval) { *istart = rank + 1; *iend = *istart; }
    else { *istart = 1; *iend = 0; }
  } else {
    int count = countval / size, remainder = countval % size;
    if (rank < remainder) { *istart = rank * (count + 1) + 1; *iend = *istart + count; }
    else { *istart = rank * count + remainder + 1; *iend = *istart + count - 1; }
  }
}

typedef struct {
  const orc_problem* pb;
  int mode, s_begin, s_end;
  long long ncell;
  double* adj_s;
  double* adj_den;
  double chi;
  double* tt_fwd;
  int* status;
  int* fwd_iters;
  int* adj_iters;
  int rc;
} orc_task;

static void* orc_worker(void* arg) {
  orc_task* t = (orc_task*)arg;
  const orc_problem* pb = t->pb;
  int maxn = 0, maxr = 1;
  for (int p = 0; p < pb->nperiod; ++p)
    if (pb->nx[p] * pb->ny[p] > maxn) maxn = pb->nx[p] * pb->ny[p];
  for (int s = t->s_begin; s < t->s_end; ++s)
    if (pb->nrec[s] > maxr) maxr = pb->nrec[s];
  double* tt = (double*)malloc(3 * (size_t)maxn * sizeof(double));
  double *adj = tt + maxn, *kden = tt + 2 * (size_t)maxn;
  double* rb = (double*)malloc(2 * (size_t)maxr * sizeof(double));
  double *tekio = rb, *wgt = rb + maxr;
  t->chi = 0;
  t->rc = ORC_OK;
  for (int s = t->s_begin; s < t->s_end; ++s) {
    int p = pb->pidx[s], nx = pb->nx[p], ny = pb->ny[p], nr = pb->nrec[s], ro = pb->rec_off[s];
    const double *xg = pb->xgrid + pb->xoff[p], *yg = pb->ygrid + pb->yoff[p];
    long long go = pb->goff[p];
    const double *sv = pb->svel + go, *m11 = pb->m11 + go, *m12 = pb->m12 + go, *m22 = pb->m22 + go;
    double chi_s = 0;
    int itf = 0, ita = 0, itd = 0;
    int st = orc_run_forward(xg, yg, nx, ny, sv, m11, m22, m12, pb->srcx[s], pb->srcy[s], nr,
                             pb->recx + ro, pb->recy + ro, pb->tt + ro, pb->weight + ro, tt,
                             tekio, &chi_s, &itf);
    if (st == ORC_OK || st == ORC_NOT_CONVERGED) {
      t->chi = t->chi + chi_s;
      if (t->tt_fwd)
        for (int i = 0; i < nr; ++i) t->tt_fwd[pb->path[ro + i]] = tekio[i];
      if (t->mode >= 2) {
        memcpy(wgt, pb->weight + ro, nr * sizeof(double));
        int sa = orc_run_adjoint(xg, yg, nx, ny, m11, m22, m12, pb->srcx[s], pb->srcy[s], nr,
                                 pb->recx + ro, pb->recy + ro, pb->tt + ro, tekio, wgt, tt, adj,
                                 &ita);
        if (sa != ORC_OK && st == ORC_OK) st = sa;
        double* ks = t->adj_s + (go - 0);
        if (t->mode == 3) {
          int sd = orc_run_adjoint_density(xg, yg, nx, ny, m11, m22, m12, pb->srcx[s],
                                           pb->srcy[s], nr, pb->recx + ro, pb->recy + ro, wgt,
                                           tt, kden, &itd);
          if (sd != ORC_OK && st == ORC_OK) st = sd;
          double* kd = t->adj_den + go;
          for (long long k = 0; k < (long long)nx * ny; ++k) {
            double v = sv[k];
            ks[k] = ks[k] + adj[k] / (v * v * v);
            kd[k] = kd[k] + kden[k] / (v * v * v);
          }
        } else {
          for (long long k = 0; k < (long long)nx * ny; ++k) {
            double v = sv[k];
            ks[k] = ks[k] + adj[k] / (v * v);
          }
        }
      }
    }
    if (st != ORC_OK && t->rc == ORC_OK) t->rc = st;
    if (t->status) t->status[s] = st;
    if (t->fwd_iters) t->fwd_iters[s] = itf;
    if (t->adj_iters) t->adj_iters[s] = ita > itd ? ita : itd;
  }
  free(tt); free(rb);
  return NULL;
}

int orc_gradient_eval_range(const orc_problem* pb, int mode, int nthreads, int s_begin,
                            int s_end, double* adj_s, double* adj_density, double* chi,
                            double* tt_fwd, int* status, int* fwd_iters, int* adj_iters) {
  if (nthreads < 1) nthreads = 1;
  long long ncell = 0;
  for (int p = 0; p < pb->nperiod; ++p) {
    long long e = pb->goff[p] + (long long)pb->nx[p] * pb->ny[p];
    if (e > ncell) ncell = e;
  }
  int count = s_end - s_begin;
  if (count < 0) return ORC_BAD_ARG;
  orc_task* tasks = (orc_task*)calloc(nthreads, sizeof(orc_task));
  pthread_t* th = (pthread_t*)calloc(nthreads, sizeof(pthread_t));
  for (int r = 0; r < nthreads; ++r) {
    int is, ie;
    orc_scatter_all_i(count, nthreads, r, &is, &ie);
    tasks[r].pb = pb;
    tasks[r].mode = mode;
    tasks[r].s_begin = s_begin + is - 1;
    tasks[r].s_end = s_begin + ie; /* exclusive */
    tasks[r].ncell = ncell;
    tasks[r].adj_s = mode >= 2 ? (double*)calloc(ncell, sizeof(double)) : NULL;
    tasks[r].adj_den = mode == 3 ? (double*)calloc(ncell, sizeof(double)) : NULL;
    tasks[r].tt_fwd = tt_fwd ? (double*)calloc(pb->npath > 0 ? pb->npath : 1, sizeof(double)) : NULL;
    tasks[r].status = status;
    tasks[r].fwd_iters = fwd_iters;
    tasks[r].adj_iters = adj_iters;
  }
  for (int r = 1; r < nthreads; ++r) pthread_create(&th[r], NULL, orc_worker, &tasks[r]);
  orc_worker(&tasks[0]);
  for (int r = 1; r < nthreads; ++r) pthread_join(th[r], NULL);
  /* reduce in rank order (MPI_Reduce to rank 0) */
  int rc = ORC_OK;
  double chi_sum = 0;
  if (adj_s) memset(adj_s, 0, ncell * sizeof(double));
  if (adj_density) memset(adj_density, 0, ncell * sizeof(double));
  if (tt_fwd) memset(tt_fwd, 0, (size_t)pb->npath * sizeof(double));
  for (int r = 0; r < nthreads; ++r) {
    chi_sum = chi_sum + tasks[r].chi;
    if (adj_s && tasks[r].adj_s)
      for (long long k = 0; k < ncell; ++k) adj_s[k] += tasks[r].adj_s[k];
    if (adj_density && tasks[r].adj_den)
      for (long long k = 0; k < ncell; ++k) adj_density[k] += tasks[r].adj_den[k];
    if (tt_fwd)
      for (int i = 0; i < pb->npath; ++i) tt_fwd[i] += tasks[r].tt_fwd[i];
    if (tasks[r].rc != ORC_OK && rc == ORC_OK) rc = tasks[r].rc;
    free(tasks[r].adj_s); free(tasks[r].adj_den); free(tasks[r].tt_fwd);
  }
  if (chi) *chi = chi_sum;
  free(tasks); free(th);
  return rc;
}

int orc_gradient_eval(const orc_problem* pb, int mode, int nthreads, double* adj_s,
                      double* adj_density, double* chi, double* tt_fwd, int* status,
                      int* fwd_iters, int* adj_iters) {
  return orc_gradient_eval_range(pb, mode, nthreads, 0, pb->nsolve, adj_s, adj_density, chi,
                                 tt_fwd, status, fwd_iters, adj_iters);
}

#ifdef ORC_COUNT_FLOPS
void orc_flop_counts(long long* out5) {
  out5[0] = cnt_visit; out5[1] = cnt_two; out5[2] = cnt_delta; out5[3] = cnt_one; out5[4] = cnt_adj;
  cnt_visit = cnt_two = cnt_delta = cnt_one = cnt_adj = 0;
}
#endif

/* ---------------------------------------------------------------------------
 * gaussian_smooth_geo_2 (src/shared/utils.f90:1194-1225), the per-period 2-D
 * kernel smoothing of tomo2d's optimize step (src/tomo2d.f90:221), with
 * gps2dist_2 (utils.f90:1280-1294) and the constants of
 * src/shared/shared_par.f90:11-15 (pi is a single-precision literal there:
 * 3.14159265359 rounded to REAL(4), then widened).  data, out: (nx, ny),
 * x fastest; lons (nx), lats (ny) in degrees, uniformly spaced; sigma in
 * degrees.  The window half-widths are the reference's integer truncations
 * nx_w = sigma3/dx and ny_w = sigma3/cosd(lat_j)/dy; cosd is evaluated as
 * cos(lat * pi/180) with the double-precision pi.  Both sums run over the
 * window in column order (i fastest), as SUM over data(m1:m2, n1:n2).
 * ------------------------------------------------------------------------- */
static double orc_gps2dist(double lat0, double lon0, double lat1, double lon1) {
  const double pi = (double)3.14159265359f;
  const double deg2rad = pi / 180.0;
  const double radius = 6371.0;
  const double dlat = (lat0 - lat1) * deg2rad;
  const double dlon = (lon1 - lon0) * deg2rad;
  const double s1 = sin(dlat * 0.5), s2 = sin(dlon * 0.5);
  const double a = s1 * s1 + s2 * s2 * cos(lat0 * deg2rad) * cos(lat1 * deg2rad);
  const double deg = 2.0 * atan2(sqrt(a), sqrt(1.0 - a));
  return radius * deg;
}

void orc_gaussian_smooth_geo_2(const double* data, int nx, int ny, const double* lons,
                               const double* lats, double sigma, double* out) {
  const double pi = (double)3.14159265359f;
  const double km2deg = 1.0 / (6371.0 * pi / 180.0);
  const double sigma3 = sigma * 3.0, sigma_sq = sigma * sigma;
  const double dx = lons[1] - lons[0], dy = lats[1] - lats[0];
  const int nxw = (int)(sigma3 / dx);
  for (int j = 0; j < ny; ++j) {
    const int nyw = (int)(sigma3 / cos(lats[j] * (3.14159265358979323846 / 180.0)) / dy);
    for (int i = 0; i < nx; ++i) {
      const int m1 = i - nxw > 0 ? i - nxw : 0, m2 = i + nxw < nx - 1 ? i + nxw : nx - 1;
      const int n1 = j - nyw > 0 ? j - nyw : 0, n2 = j + nyw < ny - 1 ? j + nyw : ny - 1;
      double swd = 0.0, sw = 0.0;
      for (int j1 = n1; j1 <= n2; ++j1)
        for (int i1 = m1; i1 <= m2; ++i1) {
          const double delta = orc_gps2dist(lats[j], lons[i], lats[j1], lons[i1]) * km2deg;
          const double w = exp(-(delta * delta) / (2.0 * sigma_sq));
          swd = swd + w * data[i1 + (size_t)nx * j1];
          sw = sw + w;
        }
      out[i + (size_t)nx * j] = (0.0 + swd) / sw;
    }
  }
}
