// smooth.cuh -- great-circle Gaussian smoothing of per-period 2-D fields,
// gaussian_smooth_geo_2 (src/shared/utils.f90:1194-1225) as tomo2d's optimize
// step applies it to every period's adj_s (src/tomo2d.f90:221).
//
// For output node (i, j) the reference sums, over the clamped window
// |i1 - i| <= nxw, |j1 - j| <= nyw(j), the weights
//   w = exp(-delta^2 / (2 sigma^2)),  delta = gps2dist(lat_j, lon_i, lat_j1, lon_i1) * km2deg
// times the data, and divides by the sum of the weights.  On the uniform
// grids the reference assumes (dx, dy from the first two nodes) w depends on
// (j, j1, |i1 - i|) only, so the GPU form evaluates each weight once per
// (period, row, window row, column offset) in a table kernel and the apply
// kernel spends one FP64 fma per window tap.  A node's weight sum depends
// on its row and on how far the window is clipped at either side, so the
// table kernel also stores, per row, the sums for every clipping, and the
// apply kernel reads its sum with one add.  The table depends on the grid
// and sigma only: callers keep it while both are unchanged.
#pragma once
#include <cuda_runtime.h>

#include <vector>

namespace sgb {

// One period's field and window geometry.
struct SmoothPeriod {
  int nx, ny;
  int nxw;      // x half-width: int(3 sigma / dx), clamped to nx - 1
  int dmax;     // min(nxw, nx - 1): largest column offset in the table
  int rows;     // window rows of the table: 2 * max_j nyw(j) + 1, clamped to ny
  int pad;
  double sigma;    // degrees
  long long goff;  // cell offset of the period's output field
  long long doff;  // cell offset of the period's input field
  long long xoff;  // offset of the period's longitudes
  long long yoff;  // offset of the period's latitudes
  long long woff;  // offset of the period's per-row nyw (it depends on sigma)
  long long toff;  // offset of the period's table (doubles)
  long long node0; // first node of the period in the apply kernel's flat numbering
};

struct SmoothArgs {
  const SmoothPeriod* per;
  int nperiod;
  const double* lons;  // degrees
  const double* lats;  // degrees
  const int* nyw;      // per (period, row): int(3 sigma / cosd(lat_j) / dy), clamped to ny - 1
  const double* data;
  double* out;
  // per (period, row), W = dmax + 1: rows x W weights w[r][d], rows x W
  // prefix sums P[r][k] = w[r][0] + ... + w[r][k], then the weight sums of a
  // node clipped to kl columns on the left and kr on the right,
  // DL[kl] + DR[kr]: DL[k] = sum_r (P[r][k] - w[r][0]), DR[k] = sum_r P[r][k].
  double* table;
  long long nodes;  // output nodes of all periods
};

// Doubles of one row's table (weights + prefix sums).
__host__ __device__ inline long long smooth_row_doubles(const SmoothPeriod& p) {
  return 2LL * (p.rows + 1) * (p.dmax + 1);
}

// Host-side geometry of one smoothing call.
struct SmoothPlan {
  std::vector<SmoothPeriod> per;
  std::vector<int> nyw;        // indexed woff + j
  long long table_doubles = 0;
  long long nyw_count = 0;     // entries of nyw
  long long nodes = 0;         // output nodes of all periods
  int max_nx = 0, max_ny = 0;
  size_t table_smem = 0;       // dynamic shared memory of the table kernel
  double taps = 0;             // window taps over all output nodes (work count)
};

// Window geometry of a set of periods, computed on the host with the same
// IEEE operations as the reference (so the integer truncations agree
// exactly).  lons / lats: host copies, per-period offsets xoff / yoff;
// goff / doff: output / input field offsets (doff NULL: the same as goff);
// sigma: one value per period.  Returns 0, or 2 (bad argument): fewer than
// 2 nodes on an axis, non-increasing or non-uniform spacing (relative 1e-9
// of the first step), sigma <= 0 or not finite, |lat| >= 90, or a grid
// whose per-row factors exceed the table kernel's shared memory.
int smooth_plan(int nperiod, const int* nx, const int* ny, const long long* goff,
                const long long* doff, const long long* xoff, const long long* yoff,
                const double* lons, const double* lats, const double* sigma, SmoothPlan* plan);

// Weight-table kernel (depends on the grid and sigma only) and apply kernel
// (one launch each) on `st`.
void launch_smooth_table(const SmoothArgs& A, const SmoothPlan& plan, cudaStream_t st);
void launch_smooth_apply(const SmoothArgs& A, const SmoothPlan& plan, cudaStream_t st);

}  // namespace sgb
