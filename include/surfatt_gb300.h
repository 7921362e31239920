/*
 * surfatt_gb300.h -- C ABI of the GB300 (sm_103a) SurfATT travel-time +
 * adjoint library (libsurfatt_gb300.so).
 *
 * Three layers, all plain C types:
 *
 *  1. Link-time drop-ins for the reference's external Fortran procedures
 *     (gfortran mangling: lower case + trailing underscore, every argument by
 *     reference, default INTEGER = 4 bytes, no hidden arguments).  Arrays are
 *     host memory, column-major (nx, ny), owned by the caller; outputs are
 *     fully overwritten.  The reference has no error return: a source on the
 *     grid boundary prints the reference's message and exits the process
 *     (as its `stop` does); every other outcome is recorded in a per-thread
 *     status readable with surfatt_last_status().
 *
 *  2. The measurement layer mirroring att_measadj (src/measadj.f90:25-114):
 *     forward + receiver interpolation + misfit, adjoint + mask, density
 *     adjoint, for one (source, period), on host buffers.
 *
 *  3. The batched engine: a whole gradient evaluation (every (period,
 *     source) solve of a work list: forward, receiver interpolation, misfit,
 *     adjoint source, one or two adjoint sweeps, mask and the per-period
 *     kernel sum) with device-resident models, in plain FP64 or with the
 *     factored unknown tau swept in FP32.
 *
 * All entry points are thread-safe; drop-in calls from different host
 * threads use separate CUDA streams and scratch buffers.
 */
#ifndef SURFATT_GB300_H
#define SURFATT_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  SURFATT_OK = 0,
  SURFATT_SOURCE_ON_BOUNDARY = 1, /* reference: 'source on the boundary, mesh error', stop */
  SURFATT_BAD_ARG = 2,            /* grid too small, point outside the grid, bad pointer */
  SURFATT_NOT_CONVERGED = 3,      /* MaxIter reached; output is the last iterate */
  SURFATT_OOM = 4,                /* device allocation failed / HBM budget exceeded */
  SURFATT_CUDA_ERROR = 5,         /* a CUDA runtime call failed */
  SURFATT_TIMEOUT = 6             /* a bounded wait gave up (serving loop) */
} surfatt_status_t;

typedef enum {
  SURFATT_PREC_FP64 = 0, /* plain FP64, reference arithmetic */
  SURFATT_PREC_FP32 = 1  /* tau swept in FP32; T0, misfit, kernels, convergence in FP64 */
} surfatt_precision_t;

typedef enum {
  SURFATT_MODE_FORWARD = 0, /* forward + misfit + synthetic times only */
  SURFATT_MODE_2D = 2,      /* tomo2d: adj_s += adj / svel^2 (src/tomo2d.f90:145-156) */
  SURFATT_MODE_3D = 3       /* tomo: adj_s += adj / svel^3, adj_density += kden / svel^3
                               (src/acqui.f90:307-316), two adjoint solves per source */
} surfatt_mode_t;

/* ---------------------------------------------------------------------------
 * 1. Drop-in symbols (src/eikon_solver_2d.f90)
 * ------------------------------------------------------------------------- */

/* replaces FSM_UW_PS_lonlat_2d, src/eikon_solver_2d.f90:764-1126 (called at
 * src/measadj.f90:68-70).  `u` is accepted and ignored, as in the reference
 * (it only feeds an error monitor that is never reported). */
void fsm_uw_ps_lonlat_2d_(const double* xx_deg, const double* yy_deg, const int* nx,
                          const int* ny, const double* spha, const double* sphb,
                          const double* sphc, double* T, const double* fun,
                          const double* x0_deg, const double* y0_deg, const double* u);

/* replaces FSM_UW_PS_cart_2d, src/eikon_solver_2d.f90:22-342 */
void fsm_uw_ps_cart_2d_(const double* xx, const double* yy, const int* nx, const int* ny,
                        const double* a, const double* b, const double* c, double* T,
                        const double* fun, const double* x0, const double* y0,
                        const double* u);

/* replaces FSM_WENO3_PS_2d (additive T = tau + T0), src/eikon_solver_2d.f90:344-548 */
void fsm_weno3_ps_2d_(const double* xx, const double* yy, const int* nx, const int* ny,
                      const double* a, const double* b, const double* c, double* T,
                      const double* fun, const double* x0, const double* y0, const double* u);

/* replaces FSM_WENO3_PS_multi_2d (T = tau * T0), src/eikon_solver_2d.f90:552-761 */
void fsm_weno3_ps_multi_2d_(const double* xx, const double* yy, const int* nx, const int* ny,
                            const double* a, const double* b, const double* c, double* T,
                            const double* fun, const double* x0, const double* y0,
                            const double* u);

/* replaces FSM_O1_JSE_lonlat_2d, src/eikon_solver_2d.f90:1276-1446 (called at
 * src/measadj.f90:85-88 and :99-102) */
void fsm_o1_jse_lonlat_2d_(const double* xx_deg, const double* yy_deg, const int* nx,
                           const int* ny, const double* spha, const double* sphb,
                           const double* sphc, const double* T, double* Ta,
                           const double* xrec_deg, const double* yrec_deg,
                           const double* sourceAdj, const int* nr);

/* replaces FSM_O1_JSE_2d, src/eikon_solver_2d.f90:1132-1273 */
void fsm_o1_jse_2d_(const double* xx, const double* yy, const int* nx, const int* ny,
                    const double* a, const double* b, const double* c, const double* T,
                    double* Ta, const double* xrec, const double* yrec,
                    const double* sourceAdj, const int* nr);

/* replaces mask, src/eikon_solver_2d.f90:1449-1467 (called at src/measadj.f90:89, :103) */
void mask_(const double* xx, const double* yy, const int* nx, const int* ny, double* TableAdj,
           const double* x0, const double* y0);

/* Status and sweep-iteration count of the calling thread's last drop-in or
 * measurement call (no counterpart in the reference, which has no status). */
int surfatt_last_status(void);
int surfatt_last_iterations(void);

/* Behaviour of a drop-in call that finds the source on the grid boundary:
 * 1 (default) prints the reference's message and exits the process like its
 * `stop`; 0 records SURFATT_SOURCE_ON_BOUNDARY and returns. */
void surfatt_set_exit_on_boundary(int enable);

/* ---------------------------------------------------------------------------
 * 2. Measurement layer (att_measadj, src/measadj.f90:62-114), host buffers
 * ------------------------------------------------------------------------- */

/* run_forward (src/measadj.f90:62-73): fun = 1/vel2d, FSM_UW_PS_lonlat_2d with
 * (m11, m22, -m12), receiver times tekio by bilinear interpolation
 * (interp2, src/shared/utils.f90:917-956), chi = 0.5*sum(w*(tekio-tt)^2).
 * Fields (nx, ny) column-major; timetable is an (nx, ny) output. */
surfatt_status_t surfatt_measadj_run_forward(const double* xgrids, const double* ygrids,
                                             int nx, int ny, const double* vel2d,
                                             const double* m11, const double* m22,
                                             const double* m12, double srcx, double srcy,
                                             int nrec, const double* recx, const double* recy,
                                             const double* tt, const double* weight,
                                             double* timetable, double* tekio, double* chi);

/* run_adjoint (src/measadj.f90:75-90): zero weight where |tekio-tt|/tt > 0.5
 * (weight updated in place), adjoint with sourceAdj = weight*(tekio-tt),
 * then mask. */
surfatt_status_t surfatt_measadj_run_adjoint(const double* xgrids, const double* ygrids,
                                             int nx, int ny, const double* m11,
                                             const double* m22, const double* m12,
                                             double srcx, double srcy, int nrec,
                                             const double* recx, const double* recy,
                                             const double* tt, const double* tekio,
                                             double* weight, const double* timetable,
                                             double* adjtable);

/* run_adjoint_density (src/measadj.f90:92-104): sourceAdj = -weight */
surfatt_status_t surfatt_measadj_run_adjoint_density(
    const double* xgrids, const double* ygrids, int nx, int ny, const double* m11,
    const double* m22, const double* m12, double srcx, double srcy, int nrec,
    const double* recx, const double* recy, const double* weight, const double* timetable,
    double* density);

/* gaussian_smooth_geo_2 (src/shared/utils.f90:1194-1225): great-circle
 * Gaussian smoothing of one (nx, ny) field, column-major, on the lon/lat grid
 * lons (nx) x lats (ny) in degrees, sigma in degrees.  Output node (i, j) is
 * sum(w * data) / sum(w) over the window |i1-i| <= int(3 sigma/dx),
 * |j1-j| <= int(3 sigma/cosd(lat_j)/dy) clamped to the grid, with
 * w = exp(-delta^2/(2 sigma^2)) and delta the gps2dist_2 distance in degrees
 * (utils.f90:1280-1294).  The reference function returns the array; the
 * binding is a subroutine writing smdata (host memory, nx*ny).  Like the
 * reference it takes dx, dy from the first two nodes and assumes uniform
 * spacing; SURFATT_BAD_ARG where the reference would read outside its
 * inputs or divide by zero: nx or ny < 2, spacing not increasing or not
 * uniform (relative 1e-9), sigma <= 0 (tomo2d rejects sigma_2d = 0,
 * src/tomo2d.f90:48-50), |lat| >= 90.  The great-circle weights depend on
 * the grid and sigma only; a host thread's call with the same nx, ny, lons,
 * lats and sigma as its previous call reuses them from the device. */
surfatt_status_t surfatt_gaussian_smooth_geo_2(const double* data, int nx, int ny,
                                               const double* lons, const double* lats,
                                               double sigma, double* smdata);

/* ---------------------------------------------------------------------------
 * Kernel combination and multigrid projection (3-D inversion)
 *
 * Layouts are the reference's arrays, Fortran order: adj_s(nperiod, nx, ny),
 * sen_*(nperiod, nx, ny, nz), vs3d(nx, ny, nz), ker(nker, nx, ny, nz),
 * xinv(nxinv, nset), gk(nxinv, nyinv, nzinv, nset).  All host memory.  The
 * results equal the reference's bit for bit (every sum in its order, every
 * product associated as written), except that the density preconditioner
 * (kdensity_coe > 0) uses the device's pow().
 * ------------------------------------------------------------------------- */

/* inv_grid_iso (src/eikon_solver_2d.f90:1541-1614): projection of the model
 * field adj(nx, ny, nz_3d) onto the nset shifted inversion grids, gk.
 * A model node that no inversion grid contains prints the reference's
 * message and ends the process (`stop`), or, with
 * surfatt_set_exit_on_boundary(0), records SURFATT_BAD_ARG. */
void inv_grid_iso_(const double* xinv, const double* yinv, const double* zinv, const int* nxinv,
                   const int* nyinv, const int* nzinv, const int* nset, const double* adj,
                   const int* nx, const int* ny, const int* nz_3d, double* gk,
                   const double* vel_x, const double* vel_y, const double* vel_z_3d);
/* inv2fwd_iso (src/eikon_solver_2d.f90:1617-1691): interpolation of gk back
 * to the model grid, summed over the sets, into update(nx, ny, nz_3d). */
void inv2fwd_iso_(const double* xinv, const double* yinv, const double* zinv, const int* nxinv,
                  const int* nyinv, const int* nzinv, const int* nset, const int* nx,
                  const int* ny, const int* nz_3d, const double* gk, const double* vel_x,
                  const double* vel_y, const double* vel_z_3d, double* update);

/* combine_kernels (src/acqui.f90:196-245, after the adj_s / adj_density
 * sums): ker(k) = -sum_p adj_s(p) * sen(p) per depth, nker = 3 with
 * use_alpha_beta_rho (rho_scaling: ker(3) = 0.33 ker(1), ker_density(3) =
 * ker_density(1)), else nker = 1 with the Brocher derivatives of vs3d / vp3d
 * (dalpha_dbeta, drho_dalpha, src/shared/utils.f90:99-145).  ker and
 * ker_density are overwritten (the reference zeroes them first,
 * src/acqui.f90:85-86). */
surfatt_status_t surfatt_combine_kernels(int nperiod, int nx, int ny, int nz, const double* adj_s,
                                         const double* adj_density, const double* sen_vs,
                                         const double* sen_vp, const double* sen_rho,
                                         const double* vs3d, const double* vp3d,
                                         int use_alpha_beta_rho, int rho_scaling, double* ker,
                                         double* ker_density);
/* post_processing_for_kernel (src/acqui.f90:247-286) for nker kernels: with
 * kdensity_coe > 0 ker(k) is preconditioned in place by its density
 * (regularize_ker_density, :288-303); then inv_grid_iso, inv2fwd_iso,
 * update / nset / chi0, and gradient_s(k) += update * weight (gradient_s is
 * read and written).  SURFATT_BAD_ARG where the reference would stop
 * because a model node lies outside the inversion grids. */
surfatt_status_t surfatt_post_process_kernels(int nker, int nx, int ny, int nz, double* ker,
                                              const double* ker_density, double kdensity_coe,
                                              const double* xinv, const double* yinv,
                                              const double* zinv, int nxinv, int nyinv,
                                              int nzinv, int nset, const double* xgrids,
                                              const double* ygrids, const double* zgrids,
                                              double chi0, double weight, double* gradient_s);
/* Both steps in one call, the kernels staying on the device in between (the
 * sequence combine_kernels, post_proc of src/tomo.f90:155-157).  ker and
 * ker_density (may be NULL) receive the combined kernels as the reference
 * leaves them (ker after preconditioning). */
surfatt_status_t surfatt_kernel_gradient(
    int nperiod, int nx, int ny, int nz, const double* adj_s, const double* adj_density,
    const double* sen_vs, const double* sen_vp, const double* sen_rho, const double* vs3d,
    const double* vp3d, int use_alpha_beta_rho, int rho_scaling, double kdensity_coe,
    const double* xinv, const double* yinv, const double* zinv, int nxinv, int nyinv, int nzinv,
    int nset, const double* xgrids, const double* ygrids, const double* zgrids, double chi0,
    double weight, double* ker, double* ker_density, double* gradient_s);
/* Device time (ms, CUDA events) of the kernels of this host thread's last
 * combine / post-process / kernel-gradient call, and their launches. */
surfatt_status_t surfatt_kernel_gradient_timing(double* kernel_ms, int* launches);

/* ---------------------------------------------------------------------------
 * The src_rec table and its work list
 *
 * One row per path: travel time, station, event, period, weight
 * (src/shared/src_rec_parser.f90:20-64).  The reference derives the
 * distinct periods (ascending), the station table (station names in order
 * of first appearance with their first coordinates, then event names that
 * are not stations) and the work list: for each station in that order that
 * is some path's event, its periods in order of first appearance, each a
 * (period, source) solve whose receivers are that event's paths at that
 * period in path order with their station's coordinates
 * (src/src_rec.f90:126-369, src/measadj.f90:39-53).  The names and periods
 * are indexed on the host once; the grouping runs on the GPU.  A period of
 * exactly 0 gets no solve, as in the reference (get_periods_by_src).
 * ------------------------------------------------------------------------- */
typedef struct surfatt_srcrec surfatt_srcrec_t;

/* Read a src_rec CSV: header row, columns tt, staname, stla, stlo, evtname,
 * evla, evlo, period (required; stel / evel ignored), weight (default 1),
 * dist (default the great-circle distance), vel (default dist / tt).
 * SURFATT_BAD_ARG for a missing file or column, a short row or a value that
 * is not a number (the reference prints and stops). */
surfatt_status_t surfatt_srcrec_read_csv(const char* fname, surfatt_srcrec_t** table);
/* The same table from arrays (names as C strings; weight may be NULL). */
surfatt_status_t surfatt_srcrec_create(int npath, const char* const* evtname,
                                       const char* const* staname, const double* stla,
                                       const double* stlo, const double* evla,
                                       const double* evlo, const double* period,
                                       const double* tt, const double* weight,
                                       surfatt_srcrec_t** table);
void surfatt_srcrec_destroy(surfatt_srcrec_t* table);
/* Sizes; nsolve is -1 before surfatt_srcrec_build_worklist. */
surfatt_status_t surfatt_srcrec_info(const surfatt_srcrec_t* table, int* npath, int* nperiod,
                                     int* nsta, int* nsolve);
surfatt_status_t surfatt_srcrec_periods(const surfatt_srcrec_t* table, double* periods);
surfatt_status_t surfatt_srcrec_stations(const surfatt_srcrec_t* table, double* stlo,
                                         double* stla);
/* Name of station i (valid while the table lives), NULL out of range. */
const char* surfatt_srcrec_station_name(const surfatt_srcrec_t* table, int i);
/* Per path: time, weight, period and the station indices of its event and
 * station and its period index (any pointer may be NULL). */
surfatt_status_t surfatt_srcrec_paths(const surfatt_srcrec_t* table, double* tt, double* weight,
                                      double* period, int* evt_station, int* station,
                                      int* period_index);
/* Build the work list on `device` (5 kernels); *nsolve receives its size. */
surfatt_status_t surfatt_srcrec_build_worklist(surfatt_srcrec_t* table, int device, int* nsolve);
/* The built work list: per solve the period index, source station, source
 * coordinates and receiver offset / count; per receiver (paths of all
 * solves, solve by solve) its coordinates, time, weight and path index --
 * the layout of surfatt_problem_t's work-list fields.  NULL skips a field. */
surfatt_status_t surfatt_srcrec_worklist(const surfatt_srcrec_t* table, int* pidx, int* sta,
                                         double* srcx, double* srcy, int* rec_off, int* nrec,
                                         double* recx, double* recy, double* tt,
                                         double* weight, int* path);
/* Device time (ms) of the last build's kernels and their count. */
surfatt_status_t surfatt_srcrec_build_timing(const surfatt_srcrec_t* table, double* kernel_ms,
                                             int* launches);
/* Write the table with the synthetic times tt_fwd (npath) as the reference
 * writes src_rec_iter files (src/src_rec.f90:285-325): the 11 columns tt,
 * staname, stla, stlo, evtname, evla, evlo, period, weight, dist, vel with
 * its F0.6 / F9.4 / F0.4 / F6.4 / F12.4 / F10.6 edits, vel = dist / tt_fwd. */
surfatt_status_t surfatt_srcrec_write_csv(const surfatt_srcrec_t* table, const char* fname,
                                          const double* tt_fwd);

/* ---------------------------------------------------------------------------
 * Surface metric from topography (curved-surface eikonal)
 * ------------------------------------------------------------------------- */

/* get_topo's per-period loop (src/grid.f90:117-145): for each period p the
 * topography topo (nx, ny, km, on the lon / lat grid of the model, degrees,
 * uniform) is smoothed by gaussian_smooth_geo_2 with sigma[p] degrees
 * (src/topo.f90:74-81), differentiated by gradient_2_geo
 * (src/shared/utils.f90:1118-1160) into fx, fy, and turned into
 * m11 = (1+fy^2)/(1+fx^2+fy^2), m22 = (1+fx^2)/(...), m12 = -fx*fy/(...)
 * and topo_angle = atand(sqrt(fx^2+fy^2)) (calc_dip_angle,
 * src/topo.f90:119-127).  Outputs (nperiod, nx, ny) Fortran order, as
 * grid.f90 stores them; any may be NULL.  SURFATT_BAD_ARG for the grids
 * and sigmas surfatt_gaussian_smooth_geo_2 rejects. */
surfatt_status_t surfatt_topo_metric(const double* topo, int nx, int ny, const double* lon,
                                     const double* lat, int nperiod, const double* sigma,
                                     double* m11, double* m22, double* m12, double* topo_angle);
/* The reference's smoothing length per period (src/grid.f90:117):
 * sigma = phase_vel * period * wavelen_factor * km2deg / (2 pi), from the
 * 1-D model's phase velocities (computed by surfdisp96 in the reference). */
surfatt_status_t surfatt_topo_sigma(int nperiod, const double* phase_vel, const double* periods,
                                    double wavelen_factor, double* sigma);
/* Device time (ms) of this host thread's last surfatt_topo_metric and its
 * kernel launches (3: weight table, smoothing, metric). */
surfatt_status_t surfatt_topo_metric_timing(double* kernel_ms, int* launches);

/* ---------------------------------------------------------------------------
 * 3. Batched gradient evaluation
 * ------------------------------------------------------------------------- */

/* A gradient evaluation's inputs.  Period p has its own lon/lat grid of
 * nx[p] x ny[p] nodes (coordinates xgrid[xoff[p]..], ygrid[yoff[p]..],
 * degrees, uniformly spaced and increasing) and fields svel (phase velocity),
 * m11, m12, m22 (surface metric, src/grid.f90:142-145), each (nx, ny)
 * column-major at cell offset goff[p].  Solve s = (period pidx[s], source
 * srcx[s]/srcy[s]) owns receivers rec_off[s] .. rec_off[s]+nrec[s]-1 of the
 * receiver table; path[r] is the receiver's index in the synthetic-time
 * table tt_fwd (npath entries) -- the reference's SrcRec%isrcs work list and
 * per-source gathers (src/src_rec.f90:252-283, 338-369).  All pointers are
 * host memory. */
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
} surfatt_problem_t;

/* Outputs of one evaluation (host buffers, any may be NULL):
 * adj_s / adj_density: ncell = goff[last] + nx*ny of the last period,
 * period-slowest; chi: sum of the solves' misfits; tt_fwd: npath synthetic
 * times; status / fwd_iters / adj_iters: per solve. */
typedef struct {
  double* adj_s;
  double* adj_density;
  double* chi;
  double* tt_fwd;
  int* status;
  int* fwd_iters;
  int* adj_iters;
} surfatt_result_t;

typedef struct surfatt_engine surfatt_engine_t;

/* Create an engine on `device`.  hbm_budget_bytes bounds the engine's device
 * allocations (0 = no bound beyond the device's free memory). */
surfatt_status_t surfatt_engine_create(surfatt_engine_t** engine, int device,
                                       size_t hbm_budget_bytes);
void surfatt_engine_destroy(surfatt_engine_t* engine);

/* Copy a problem to the device (grids, fields, work list, receivers) and size
 * the engine's workspace.  Replaces any previously loaded problem. */
surfatt_status_t surfatt_engine_load(surfatt_engine_t* engine, const surfatt_problem_t* pb);

/* Replace the phase-velocity fields of the loaded problem (a line-search
 * trial model or the next inversion iterate); same layout as pb->svel. */
surfatt_status_t surfatt_engine_update_velocity(surfatt_engine_t* engine, const double* svel);

/* Launch one gradient evaluation on the engine's stream (asynchronous).
 * SURFATT_PREC_FP32 runs, unless surfatt_engine_set_kernel or the autotuner
 * chose otherwise, the row-per-lane kernel: one warp per solve on grids of
 * at most 128 rows, a team of 2 - 4 warps per solve up to 512 rows (taller
 * or wider than 4096 columns: one block per solve).  A batch that mixes
 * grid heights runs as one launch per team class, concurrently on the
 * engine's side streams; each solve's results are the same as alone. */
surfatt_status_t surfatt_engine_run(surfatt_engine_t* engine, surfatt_mode_t mode,
                                    surfatt_precision_t precision);

/* Wait for the last run; returns its overall status (first failing solve). */
surfatt_status_t surfatt_engine_sync(surfatt_engine_t* engine);

/* Copy the last run's results to host buffers (synchronises first). */
surfatt_status_t surfatt_engine_results(surfatt_engine_t* engine, surfatt_result_t* out);

/* Device time of the last run (ms, CUDA events on the engine's stream) and of
 * its solve kernel alone; number of kernel launches it issued. */
surfatt_status_t surfatt_engine_timing(surfatt_engine_t* engine, double* total_ms,
                                       double* solve_kernel_ms, int* launches);

/* Kernel smoothing of tomo2d's optimize step (src/tomo2d.f90:203-233, the
 * loop at :216-222): ker_s of period p = gaussian_smooth_geo_2(adj_s of
 * period p, its lon/lat axes, sigma) for every period of the last run's
 * adj_s (mode 2 or 3), computed on the device from the engine's resident
 * adj_s.  ker_s (host, ncell doubles, the adj_s layout) may be NULL: the
 * smoothing is then only enqueued (surfatt_engine_sync waits for it) and the
 * result stays on the device.  The weight table is built on the first call
 * after a load or a change of sigma and kept for later calls (an inversion
 * smooths every iteration's adj_s on the same grids with the same sigma).
 * SURFATT_BAD_ARG before a mode-2/3 run and for the arguments
 * surfatt_gaussian_smooth_geo_2 rejects. */
surfatt_status_t surfatt_engine_smooth(surfatt_engine_t* engine, double sigma, double* ker_s);
/* Device time (ms) of the last surfatt_engine_smooth, its window taps over
 * all output nodes, and its kernel launches (2 when it built the weight
 * table, else 1: apply only). */
surfatt_status_t surfatt_engine_smooth_timing(surfatt_engine_t* engine, double* kernel_ms,
                                              double* taps, int* launches);

/* Launch configuration of the last run's solve kernel: blocks, threads per
 * block, resident blocks per SM, dynamic shared memory per block. */
surfatt_status_t surfatt_engine_launch_config(surfatt_engine_t* engine, int* grid, int* block,
                                              int* blocks_per_sm, size_t* smem_bytes);

/* Time every solve-kernel variant that applies to the loaded problem (plain
 * FP64: 0 solves cut into work items, 1 whole solves; FP32: the
 * row-per-lane kernel's variants -- 0 / 1: cell constants loaded a step
 * ahead, 8 resident warps per SM, solves cut into work items / whole; 2 / 3:
 * cell constants loaded at the visit, 12 / 8 warps, items / whole; 4 / 5, on
 * grids of more than 128 rows only: the tall grids swept by one warp in
 * 128-row strips instead of a team of warps (same results), items (the
 * whole forward, then one per adjoint field) / whole solves --
 * and the block-per-solve kernel) with one warm-up and one timed evaluation each,
 * and use the fastest for later runs of this precision until the next load.
 * Returns the chosen kernel (0 FP64, 1 FP32 block, 2 FP32 warp), its variant
 * and its solve-kernel time. */
surfatt_status_t surfatt_engine_autotune(surfatt_engine_t* engine, surfatt_mode_t mode,
                                         surfatt_precision_t precision, int* kind, int* variant,
                                         double* best_ms);
/* Choose the solve kernel of later runs at `precision` by hand (as
 * surfatt_engine_autotune would): kind (0 FP64, 1 FP32 block, 2 FP32 warp)
 * and variant (as above); -1 leaves a field automatic.  A kernel that does
 * not apply to the loaded grids makes the next run return
 * SURFATT_BAD_ARG. */
surfatt_status_t surfatt_engine_set_kernel(surfatt_engine_t* engine, surfatt_precision_t precision,
                                          int kind, int variant);
/* Per-phase SM cycle counters of the FP32 warp kernel (default: off).  When
 * on, every run sums clock64() intervals per solve phase over all solves:
 * [0] source cell + T0, [1] forward sweeps, [2] receiver times + misfit,
 * [3] adjoint coefficients + sources, [4] adjoint sweeps, [5] mask + kernel
 * slot; surfatt_engine_phase_cycles copies the six sums of the last run. */
surfatt_status_t surfatt_engine_set_profile(surfatt_engine_t* engine, int enable);
surfatt_status_t surfatt_engine_phase_cycles(surfatt_engine_t* engine, double* cycles);
/* Kernel and variant used by the last run. */
surfatt_status_t surfatt_engine_kernel_variant(surfatt_engine_t* engine, int* kind, int* variant);

/* Capture each (mode, precision) evaluation -- resets, solve kernel, kernel
 * sums, misfit sum -- into a CUDA graph on its first run and replay it with
 * one graph launch afterwards (default: on).  A load, or a buffer that had to
 * grow, makes the next run capture again; a velocity update does not. */
surfatt_status_t surfatt_engine_set_graphs(surfatt_engine_t* engine, int enable);

/* Keep every solve's travel-time field T = tau*T0 of later runs (default
 * off; forward grids of the solves one after another, solve s at the offset
 * of its kernel slot: sum over the solves before it of nx*ny of their
 * periods), and copy the last run's fields to `T` (host, that many doubles).
 * The fields are what FSM_UW_PS_lonlat_2d returns per solve
 * (src/eikon_solver_2d.f90:1124; src/measadj.f90:68-70), for checks of the
 * whole field rather than its receiver values.  A solve that failed has a
 * zero field. */
surfatt_status_t surfatt_engine_set_keep_fields(surfatt_engine_t* engine, int enable);
surfatt_status_t surfatt_engine_fields(surfatt_engine_t* engine, double* T);

/* Test hook of the bounded device wait (no counterpart in the reference;
 * default solve = -1: off).  With the FP32 row kernel cutting solves into
 * work items, the first item of `solve` is skipped without being marked
 * done, so the solve's next item waits for it until wait_polls polls (0:
 * the production limit of 2^24) have run out; the solve then ends with
 * SURFATT_TIMEOUT and contributes nothing, every other solve completes.
 * The wait is the one a real stall of a previous item would meet; nothing
 * on the device faults or hangs. */
surfatt_status_t surfatt_engine_test_hold(surfatt_engine_t* engine, int solve, int wait_polls);

/* Device addresses of the last run's results as they sit in the engine's
 * memory: adj_s and adj_density (ncell doubles, the problem's per-period
 * layout; NULL when the mode does not produce them), tt_fwd (npath doubles)
 * and chi (one double), and the engine's stream (a cudaStream_t) that wrote
 * them.  They stay valid until the next load.  For a caller that reduces the
 * results of several ranks on the device (the MPI_Reduce of adj_s,
 * adj_density, chi and the synthetic-time table, src/acqui.f90:152-160,
 * 205-206) without copying them to the host; order the reduction after the
 * run (surfatt_engine_sync, or an event on the stream). */
surfatt_status_t surfatt_engine_device_results(surfatt_engine_t* engine, double** adj_s,
                                               double** adj_density, double** tt_fwd,
                                               double** chi, void** stream);

/* Total sweep cell visits of the last run (forward, adjoint), for the
 * algorithmic roofline. */
surfatt_status_t surfatt_engine_work(surfatt_engine_t* engine, double* fwd_cell_updates,
                                     double* adj_cell_updates);

/* FP64 and FP32 FMA issue peaks of `device` in TFLOP/s (an FMA = 2 flops),
 * measured with independent FMA chains (about 0.1 s).  No counterpart in the
 * reference: these are the denominators of the sweep kernels' roofline. */
surfatt_status_t surfatt_measure_peaks(int device, double* fp64_tflops, double* fp32_tflops);

/* FSM_UW_PS_lonlat_2d on device arrays without allocating any memory.
 * No counterpart in the reference.  For callers that must not allocate
 * device memory when they call the solver (a host framework whose memory
 * pool owns the HBM, or a loop that cannot afford the device-wide
 * synchronisation of cudaMalloc/cudaFree).  All arrays are device pointers
 * with the drop-in's layout; T (nx, ny) receives the travel times and
 * status_iters[0..1] (device ints) the status and sweep iterations.  The
 * solve is enqueued on `stream` (a cudaStream_t, NULL = default stream) and
 * the call returns without waiting.  Scratch is a fixed array inside the
 * library (about 4.8 MB per GPU, held until the process exits): grids above
 * 16384 cells or 2048 nodes per axis are rejected with SURFATT_BAD_ARG.  The
 * first call on a device looks up the scratch address and should come
 * before any stream capture; the address is kept for the process, so the
 * entry point must not be called after cudaDeviceReset on that device.
 * Calls share the scratch: calls that overlap on the GPU race and must be
 * ordered (one stream, or events).  The return value is this launch's own
 * error only (an error pending from earlier work is left untouched). */
surfatt_status_t surfatt_uw_lonlat_solve_noalloc(const double* xx_deg, const double* yy_deg,
                                                 int nx, int ny, const double* spha,
                                                 const double* sphb, const double* sphc,
                                                 const double* fun, double x0_deg, double y0_deg,
                                                 double* T, int* status_iters, void* stream);

/* ---------------------------------------------------------------------------
 * 4. Serving loop (no counterpart in the reference, whose drivers call the
 *    path synchronously): requests -- gradient evaluations, line-search
 *    trial models, forward-only runs -- admitted by an HBM budget and run
 *    concurrently, with models and station tables resident on the device.
 * ------------------------------------------------------------------------- */
typedef struct surfatt_server surfatt_server_t;

typedef struct {
  long long submitted, completed, failed, solves;
  double p50_ms, p99_ms, mean_ms; /* submit -> result ready, per request */
  double span_s;                  /* first submit -> last completion */
  double solves_per_s;            /* solves completed / span */
  size_t hbm_budget_bytes, hbm_peak_bytes;
  int inflight_peak;
} surfatt_server_stats_t;

/* A server on `device` owning one device allocation of hbm_budget_bytes
 * (every model, work list and in-flight request lives in it) and running at
 * most max_inflight requests at a time. */
surfatt_status_t surfatt_server_create(surfatt_server_t** server, int device,
                                       size_t hbm_budget_bytes, int max_inflight);
/* Waits for running requests, drops queued ones, frees everything. */
void surfatt_server_destroy(surfatt_server_t* server);
/* Make the periods of `pb` (grids, metric m11/m12/m22, velocity) resident. */
surfatt_status_t surfatt_server_add_model(surfatt_server_t* server, const surfatt_problem_t* pb,
                                          int* model_id);
/* Make the work list of `pb` (solves, receivers, observed times, weights,
 * path indices) resident, for the periods of model `model_id`. */
surfatt_status_t surfatt_server_add_worklist(surfatt_server_t* server, int model_id,
                                             const surfatt_problem_t* pb, int* worklist_id);
/* Queue an evaluation of a work list; `svel` (may be NULL: the model's
 * velocity) is a velocity model laid out like pb->svel, copied at submit. */
surfatt_status_t surfatt_server_submit(surfatt_server_t* server, int worklist_id,
                                       const double* svel, surfatt_mode_t mode,
                                       surfatt_precision_t precision, long long* ticket);
/* Wait (timeout_s <= 0: no limit) for a request, copy its results into
 * `out` (host buffers; NULL members are skipped) and release it. */
surfatt_status_t surfatt_server_wait(surfatt_server_t* server, long long ticket,
                                     double timeout_s, surfatt_result_t* out,
                                     double* latency_ms);
surfatt_status_t surfatt_server_stats(surfatt_server_t* server, surfatt_server_stats_t* stats);
surfatt_status_t surfatt_server_reset_stats(surfatt_server_t* server);

/* Library version string. */
const char* surfatt_version(void);

#ifdef __cplusplus
}
#endif
#endif
