// project.cuh -- kernel combination and multigrid projection of SurfATT's
// 3-D inversion: combine_kernels (src/acqui.f90:196-245),
// post_processing_for_kernel (src/acqui.f90:247-286) with
// regularize_ker_density (:288-303), inv_grid_iso / inv2fwd_iso
// (src/eikon_solver_2d.f90:1541-1691).
//
// Every sum keeps the reference's order and every product its association,
// with explicitly rounded FP64 operations, so the results are the
// reference's bit for bit (the density preconditioner's pow() aside).
//
// The reference locates each model node in each inversion grid with a
// walking search whose state carries over from node to node
// (locate_within_cube, :1470-1538).  The cell it finds is unique except
// when a node lies exactly on an inversion-grid plane; there the walk's
// direction decides between the lower cell (weight 1) and the upper one
// (weight 0), and that choice changes the order of inv2fwd_iso's eight-term
// sum.  The loops walk upwards except at the first node of a row (x) or
// column (z) after the first, which the walk reaches from above.  The host
// computes both resolutions per coordinate (`lo`: walk up from cell 1, `up`:
// walk down from the last cell) and the kernels pick one by that rule.
#pragma once
#include <cuda_runtime.h>

#include <vector>

namespace sgb {

// Locations of one axis's model coordinates in one axis's inversion grids,
// for every set: cell[(s*2 + u)*n + i] (0-based cell, -1 outside) and its
// weight w, u = 0 walking up, u = 1 walking down.  rng[s*ninv + a] = first
// and last interior model node (1..n-2) that has inversion node a as a
// corner of a cell it may be assigned to (first > last: none).
struct ProjAxis {
  int n, ninv;
  std::vector<int> cell;
  std::vector<double> w;
  std::vector<int2> rng;
};

struct ProjPlan {
  int nx = 0, ny = 0, nz = 0, nset = 0;
  double dx = 0, dy = 0, dz = 0;  // vel_x(2)-vel_x(1), ... (:1559-1561)
  ProjAxis ax[3];
  // First node (in the reference's loop order) that cannot be located, as
  // the reference reports it before stopping: which projection (1 inv_grid_iso,
  // 2 inv2fwd_iso, 0 none) and its coordinates.
  int bad = 0;
  double bad_xyz[3] = {0, 0, 0};
};

// Host plan.  Returns 0, 2 (bad argument: an axis with fewer than 2 model
// nodes or inversion nodes or more than 1024 inversion nodes, nset < 1) or 7
// (a node cannot be located; plan.bad says where).  `need` selects the projections that must locate their nodes:
// bit 0 inv_grid_iso (interior nodes), bit 1 inv2fwd_iso (all nodes).
int proj_plan(const double* xinv, const double* yinv, const double* zinv, int nxinv, int nyinv,
              int nzinv, int nset, const double* vx, const double* vy, const double* vz, int nx,
              int ny, int nz, int need, ProjPlan* plan);

// Device copy of a plan's tables.
struct ProjDev {
  int nx, ny, nz, nset;
  int ninv[3];
  double dx, dy, dz;
  const int* cell[3];
  const double* w[3];
  const int2* rng[3];
};

// Doubles / ints / int2 of the device tables of a plan, and the host-side
// packing of them (cells, weights, ranges: x then y then z).
struct ProjTables {
  std::vector<int> cells;
  std::vector<double> w;
  std::vector<int2> rng;
  long long cell_off[3], w_off[3], rng_off[3];
};
void proj_pack(const ProjPlan& plan, ProjTables* t);
ProjDev proj_dev(const ProjPlan& plan, const ProjTables& t, const int* d_cells,
                 const double* d_w, const int2* d_rng);

// combine_kernels on the device.  adj_s / adj_density (P, nx, ny), sen_*
// (P, nx, ny, nz), vs3d / vp3d (nx, ny, nz), ker / ker_density
// (nker, nx, ny, nz), nker = use_alpha_beta_rho ? 3 : 1.  Overwrites ker and
// ker_density (the reference zeroes them first, src/acqui.f90:85-86).
void launch_combine(int P, int nx, int ny, int nz, const double* adj_s,
                    const double* adj_density, const double* sen_vs, const double* sen_vp,
                    const double* sen_rho, const double* vs3d, const double* vp3d,
                    int use_alpha_beta_rho, int rho_scaling, double* ker, double* ker_density,
                    cudaStream_t st);

// Scratch of inv_grid_iso's two passes for nker kernels: the eight terms of
// every (set, interior node) and its packed cell.
inline size_t proj_terms_doubles(const ProjPlan& p, int nker) {
  return (size_t)nker * p.nset * 8 * (size_t)(p.nx - 2) * (p.ny - 2) * (p.nz - 2);
}
inline size_t proj_cells_ints(const ProjPlan& p) {
  return (size_t)p.nset * (size_t)(p.nx - 2) * (p.ny - 2) * (p.nz - 2);
}

// post_processing_for_kernel on the device for nker kernels: density
// preconditioning of ker in place when kdensity_coe > 0, the scaled kernel
// A = ker*dx*dy*dz into `scaled` (nker*N3), inv_grid_iso into gk
// (nker * nset * ninv) through `terms` / `cells` (proj_terms_doubles /
// proj_cells_ints), inv2fwd_iso, update / nset / chi0, gradient_s +=
// update * weight.  absmax: nker unsigned long long of scratch.  4 launches
// (+2 with preconditioning: a memset and the density maximum).
void launch_post_process(const ProjDev& P, int nker, double* ker, const double* ker_density,
                         double kdensity_coe, double* scaled, double* terms, int* cells,
                         double* gk, unsigned long long* absmax, double chi0, double weight,
                         double* gradient_s, cudaStream_t st);

// The two projections alone (the drop-in subroutines): inv_grid_iso of one
// field adj (nx, ny, nz) into gk (nset * ninv), and inv2fwd_iso of gk into
// update (nx, ny, nz).  `scaled`: N3 doubles of scratch; terms / cells as
// above for one kernel.
void launch_inv_grid(const ProjDev& P, const double* adj, double* scaled, double* terms,
                     int* cells, double* gk, cudaStream_t st);
void launch_inv2fwd(const ProjDev& P, const double* gk, double* update, cudaStream_t st);

}  // namespace sgb
