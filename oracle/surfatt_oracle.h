/*
 * surfatt_oracle.h -- CPU oracle for the SurfATT travel-time + adjoint path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * Fortran (SurfATT 1.6.1, src/eikon_solver_2d.f90, src/measadj.f90,
 * src/shared/utils.f90 interp2, src/acqui.f90 / src/tomo2d.f90 kernel
 * accumulation).  It is the parity checker for the CUDA library and the timed
 * CPU baseline.  Only tests, the smoke check and the benchmark's CPU-baseline
 * leg may load it; the product library never links or calls it.
 *
 * Parity status: UNPINNED by the reference's own tests.  The reference ships
 * no unit tests, golden vectors or known-answer tests for this path, and it
 * cannot be compiled in this environment (no Fortran compiler).  The oracle is
 * pinned instead by analytic known-answer tests (homogeneous medium),
 * reciprocity and a finite-difference check of the adjoint gradient.
 *
 * Conventions (Fortran, kept): arrays are column-major (nx, ny), i.e. element
 * (ix, iy) with 0-based ix, iy lives at [ix + nx*iy]; x (longitude) fastest.
 * The routines reproduce the reference's implicit REAL(4) variables
 * (r1, r2, sigx, sigy, coe), its single-rounded literal constants
 * (pi, tol, eps) and its loop orders.
 */
#ifndef SURFATT_ORACLE_H
#define SURFATT_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ORC_OK = 0,
  ORC_SOURCE_ON_BOUNDARY = 1, /* reference: 'source on the boundary, mesh error' + stop */
  ORC_BAD_ARG = 2,            /* point outside the grid, nx/ny < 4, ... */
  ORC_NOT_CONVERGED = 3       /* MaxIter reached (the reference continues silently) */
};

/* ---- A1: FSM_UW_PS_lonlat_2d (src/eikon_solver_2d.f90:764-1126) ---- */
int orc_fsm_uw_ps_lonlat_2d(const double* xx_deg, const double* yy_deg, int nx, int ny,
                            const double* spha, const double* sphb, const double* sphc,
                            double* T, const double* fun, double x0_deg, double y0_deg,
                            int* niter);
/* FSM_UW_PS_cart_2d (src/eikon_solver_2d.f90:22-342): same sweep, Cartesian T0 */
int orc_fsm_uw_ps_cart_2d(const double* xx, const double* yy, int nx, int ny,
                          const double* a, const double* b, const double* c,
                          double* T, const double* fun, double x0, double y0, int* niter);
/* ---- A7: FSM_WENO3_PS_multi_2d (src/eikon_solver_2d.f90:552-761) ---- */
int orc_fsm_weno3_ps_multi_2d(const double* xx, const double* yy, int nx, int ny,
                              const double* a, const double* b, const double* c,
                              double* T, const double* fun, double x0, double y0, int* niter);
/* ---- A8: FSM_WENO3_PS_2d (src/eikon_solver_2d.f90:344-548) ---- */
int orc_fsm_weno3_ps_2d(const double* xx, const double* yy, int nx, int ny,
                        const double* a, const double* b, const double* c,
                        double* T, const double* fun, double x0, double y0, int* niter);

/* ---- A2: FSM_O1_JSE_lonlat_2d (src/eikon_solver_2d.f90:1276-1446) ---- */
int orc_fsm_o1_jse_lonlat_2d(const double* xx_deg, const double* yy_deg, int nx, int ny,
                             const double* spha, const double* sphb, const double* sphc,
                             const double* T, double* Ta, const double* xrec_deg,
                             const double* yrec_deg, const double* sourceAdj, int nr,
                             int* niter);
/* FSM_O1_JSE_2d (src/eikon_solver_2d.f90:1132-1273) */
int orc_fsm_o1_jse_2d(const double* xx, const double* yy, int nx, int ny,
                      const double* a, const double* b, const double* c,
                      const double* T, double* Ta, const double* xrec,
                      const double* yrec, const double* sourceAdj, int nr, int* niter);

/* ---- A3: mask (src/eikon_solver_2d.f90:1449-1467) ---- */
void orc_mask(const double* xx, const double* yy, int nx, int ny, double* TableAdj,
              double x0, double y0);

/* ---- interp2_0_dp (src/shared/utils.f90:917-942); returns ORC_BAD_ARG when
 *      the query point has no grid node above it in x or y ---- */
int orc_interp2(const double* x, int nx, const double* y, int ny, const double* v,
                double xq, double yq, double* vq);

/* ---- A4/A5: att_measadj (src/measadj.f90:62-104) ---- */
int orc_run_forward(const double* xgrids, const double* ygrids, int nx, int ny,
                    const double* vel2d, const double* m11, const double* m22,
                    const double* m12, double srcx, double srcy, int nrec,
                    const double* recx, const double* recy, const double* tt,
                    const double* weight, double* timetable, double* tekio, double* chi,
                    int* niter);
/* weight is updated in place (outlier zeroing, measadj.f90:82-84) */
int orc_run_adjoint(const double* xgrids, const double* ygrids, int nx, int ny,
                    const double* m11, const double* m22, const double* m12,
                    double srcx, double srcy, int nrec, const double* recx,
                    const double* recy, const double* tt, const double* tekio,
                    double* weight, const double* timetable, double* adjtable, int* niter);
int orc_run_adjoint_density(const double* xgrids, const double* ygrids, int nx, int ny,
                            const double* m11, const double* m22, const double* m12,
                            double srcx, double srcy, int nrec, const double* recx,
                            const double* recy, const double* weight,
                            const double* timetable, double* density, int* niter);

/* ---- A6 + the per-(source, period) loop (src/acqui.f90:91-161, 307-316;
 *      src/tomo2d.f90:145-201) ----
 *
 * One gradient evaluation over a work list of (period, source) solves.
 * Period p has its own grid: nx[p] x ny[p] nodes, coordinates
 * xgrid[xoff[p] .. xoff[p]+nx[p]), ygrid[yoff[p] .. ], fields svel/m11/m12/m22
 * at cell offset goff[p] (each (nx, ny) column-major).  Solve s uses period
 * pidx[s], source (srcx[s], srcy[s]) and receivers rec_off[s] ..
 * rec_off[s]+nrec[s]-1 of the receiver table (recx, recy, tt, weight, path).
 * mode 2: 2-D tomography (tomo2d.f90): adj_s += adj / svel^2, one adjoint.
 * mode 3: 3-D tomography (acqui.f90): adj_s += adj / svel^3 and
 *         adj_density += kden / svel^3 (two adjoints per solve).
 * mode 0: forward only (chi and tt_fwd only).
 * The work list is split over `nthreads` threads in contiguous blocks exactly
 * like scatter_all_i (src/shared/parallel.f90:1877-1903); per-thread partial
 * kernels are summed in thread order.
 * Outputs: adj_s / adj_density (sum over periods of nx*ny, zeroed first),
 * chi (scalar), tt_fwd[path] (npath entries, zeroed first), per-solve status
 * and iteration counts (may be NULL).  `weight` is not modified. */
typedef struct {
  int nperiod;
  const int* nx;
  const int* ny;
  const long long* xoff;
  const long long* yoff;
  const long long* goff;
  const double* xgrid;
  const double* ygrid;
  const double* svel;
  const double* m11;
  const double* m12;
  const double* m22;
  int nsolve;
  const int* pidx;
  const double* srcx;
  const double* srcy;
  const int* rec_off;
  const int* nrec;
  const double* recx;
  const double* recy;
  const double* tt;
  const double* weight;
  const int* path;
  int npath;
} orc_problem;

int orc_gradient_eval(const orc_problem* pb, int mode, int nthreads, double* adj_s,
                      double* adj_density, double* chi, double* tt_fwd, int* status,
                      int* fwd_iters, int* adj_iters);

/* The same loop restricted to solves [s_begin, s_end): used to time a bounded
 * sample and by the multi-rank tests (each rank owns a contiguous block). */
int orc_gradient_eval_range(const orc_problem* pb, int mode, int nthreads, int s_begin,
                            int s_end, double* adj_s, double* adj_density, double* chi,
                            double* tt_fwd, int* status, int* fwd_iters, int* adj_iters);

/* scatter_all_i (src/shared/parallel.f90:1877-1903), 1-based istart/iend */
void orc_scatter_all_i(int countval, int size, int rank, int* istart, int* iend);

/* gaussian_smooth_geo_2 (src/shared/utils.f90:1194-1225) of one (nx, ny)
 * field, x fastest; lons / lats in degrees (uniform), sigma in degrees. */
void orc_gaussian_smooth_geo_2(const double* data, int nx, int ny, const double* lons,
                               const double* lats, double sigma, double* out);

/* Kernel combination and multigrid projection (oracle_project.c):
 * combine_kernels (src/acqui.f90:196-245), inv_grid_iso / inv2fwd_iso
 * (src/eikon_solver_2d.f90:1541-1691), post_processing_for_kernel
 * (src/acqui.f90:247-286), get_inv_grids (src/model.f90:127-172).  The
 * projections return 1 (and the coordinates in bad[3]) where the reference
 * prints "I cannot locate the receiver in the domain." and stops. */
double orc_dalpha_dbeta_1(double vs);
double orc_drho_dalpha_1(double vp);
void orc_combine_kernels(int P, int nx, int ny, int nz, const double* adj_s,
                         const double* adj_density, const double* sen_vs, const double* sen_vp,
                         const double* sen_rho, const double* vs3d, const double* vp3d,
                         int use_alpha_beta_rho, int rho_scaling, double* ker,
                         double* ker_density);
int orc_inv_grid_iso(const double* xinv, const double* yinv, const double* zinv, int nxinv,
                     int nyinv, int nzinv, int nset, const double* adj, int nx, int ny, int nz,
                     double* gk, const double* vx, const double* vy, const double* vz,
                     double* bad);
int orc_inv2fwd_iso(const double* xinv, const double* yinv, const double* zinv, int nxinv,
                    int nyinv, int nzinv, int nset, int nx, int ny, int nz, const double* gk,
                    const double* vx, const double* vy, const double* vz, double* update,
                    double* bad);
int orc_post_process_kernels(int nker, int nx, int ny, int nz, double* ker,
                             const double* ker_density, double kdensity_coe, const double* xinv,
                             const double* yinv, const double* zinv, int nxinv, int nyinv,
                             int nzinv, int nset, const double* xgrids, const double* ygrids,
                             const double* zgrids, double chi0, double weight, double* gradient_s,
                             double* bad);
void orc_get_inv_grids(const double* xgrids, int nx, const double* ygrids, int ny,
                       const double* zgrids, int nz, int ninvx, int ninvy, int ninvz, int nset,
                       double* xinv, double* yinv, double* zinv);

/* Work list and receiver gathers from a src_rec table (oracle_srcrec.c):
 * get_periods, get_sta, scatter_src_gather, get_periods_by_src,
 * get_evt_gather, get_sta_pos (src/src_rec.f90:126-369).  0-based outputs;
 * capacities: periods npath, stations 2*npath, solves and receivers npath.
 * weight may be NULL (all ones). */
int orc_srcrec_worklist(int npath, const char* const* evtname, const char* const* staname,
                        const double* stla, const double* stlo, const double* evla,
                        const double* evlo, const double* period, const double* tt,
                        const double* weight, int* nperiod_out, double* periods,
                        int* nsta_out, const char** sta_name, double* sta_lo, double* sta_la,
                        int* nsolve_out, int* pidx, int* sta, double* srcx, double* srcy,
                        int* rec_off, int* nrec, double* recx, double* recy, double* rtt,
                        double* rweight, int* rpath);

/* Surface metric from topography (oracle_topo.c): gradient_2_geo
 * (src/shared/utils.f90:1118-1160) and get_topo's per-period loop
 * (src/grid.f90:117-145).  Metric outputs (nperiod, nx, ny), period
 * fastest; any may be NULL. */
void orc_gradient_2_geo(const double* f, int nx, int ny, const double* lon, const double* lat,
                        double* tx, double* ty);
int orc_topo_metric(const double* topo, int nx, int ny, const double* lon, const double* lat,
                    int nperiod, const double* sigma, double* m11, double* m22, double* m12,
                    double* angle);

#ifdef __cplusplus
}
#endif
#endif
