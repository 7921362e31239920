// smooth.cu -- great-circle Gaussian smoothing of per-period fields
// (gaussian_smooth_geo_2, src/shared/utils.f90:1194-1225): window plan on the
// host, a weight-table kernel and a one-fma-per-tap apply kernel.
#include <cmath>

#include "common.cuh"
#include "smooth.cuh"

namespace sgb {

namespace {

// Constants of src/shared/shared_par.f90:11-15 (pi is a default-real literal
// widened to double; the others are double expressions of it).
constexpr double kDeg2Rad = PI_S / 180.0;
constexpr double kKm2Deg = 1.0 / (6371.0 * PI_S / 180.0);
constexpr double kRadius = 6371.0;
// cosd() of the window height, evaluated as cos(x * pi / 180) with the
// double-precision pi.
constexpr double kCosdScale = 3.14159265358979323846 / 180.0;
constexpr size_t kTableSmemMax = 200 * 1024;

bool uniform_axis(const double* x, int n, double step) {
  for (int k = 1; k < n; ++k) {
    const double d = x[k] - x[k - 1];
    if (!std::isfinite(x[k]) || !(std::fabs(d - step) <= 1e-9 * step)) return false;
  }
  return std::isfinite(x[0]);
}

}  // namespace

int smooth_plan(int nperiod, const int* nx, const int* ny, const long long* goff,
                const long long* doff, const long long* xoff, const long long* yoff,
                const double* lons, const double* lats, const double* sigma, SmoothPlan* plan) {
  SmoothPlan& P = *plan;
  P = SmoothPlan();
  if (nperiod < 0) return ST_BAD_ARG;
  P.per.resize(nperiod);
  for (int p = 0; p < nperiod; ++p) {
    if (!std::isfinite(sigma[p]) || !(sigma[p] > 0.0)) return ST_BAD_ARG;
    const double sigma3 = sigma[p] * 3;  // utils.f90:1205
    const int X = nx[p], Y = ny[p];
    if (X < 2 || Y < 2) return ST_BAD_ARG;  // dx, dy read the first two nodes
    const double* lo = lons + xoff[p];
    const double* la = lats + yoff[p];
    const double dx = lo[1] - lo[0], dy = la[1] - la[0];  // :1209-1210
    if (!(dx > 0.0) || !(dy > 0.0) || !uniform_axis(lo, X, dx) || !uniform_axis(la, Y, dy))
      return ST_BAD_ARG;
    for (int j = 0; j < Y; ++j)
      if (!(std::fabs(la[j]) < 90.0)) return ST_BAD_ARG;
    // nx = sigma3/dx (:1211): truncation of the quotient; clamped to the grid
    // (the window is clamped to it anyway, :1216).
    const double vx = sigma3 / dx;
    const int nxw = vx >= (double)(X - 1) ? X - 1 : (int)vx;
    const long long woff = (long long)P.nyw.size();
    P.nyw.resize(woff + Y, 0);
    int wmax = 0;
    // columns summed over a row's nodes: sum_i (min(nxw, i) + min(nxw, X-1-i) + 1)
    const double side = nxw >= X - 1 ? 0.5 * (double)X * (X - 1)
                                     : 0.5 * nxw * (nxw + 1.0) + (double)(X - 1 - nxw) * nxw;
    const double cols = 2.0 * side + X;
    for (int j = 0; j < Y; ++j) {
      const double vy = sigma3 / std::cos(la[j] * kCosdScale) / dy;  // :1213
      const int w = vy >= (double)(Y - 1) ? Y - 1 : (int)vy;
      P.nyw[woff + j] = w;
      wmax = w > wmax ? w : wmax;
      const int nr = (j + w < Y - 1 ? j + w : Y - 1) - (j - w > 0 ? j - w : 0) + 1;
      P.taps += (double)nr * cols;
    }
    SmoothPeriod& s = P.per[p];
    s.nx = X;
    s.ny = Y;
    s.nxw = nxw;
    s.dmax = nxw;
    s.rows = 2 * wmax + 1 < Y ? 2 * wmax + 1 : Y;
    s.pad = 0;
    s.sigma = sigma[p];
    s.goff = goff[p];
    s.doff = doff ? doff[p] : goff[p];
    s.xoff = xoff[p];
    s.yoff = yoff[p];
    s.woff = woff;
    s.toff = P.table_doubles;
    s.node0 = P.nodes;
    P.table_doubles += (long long)Y * smooth_row_doubles(s);
    P.nodes += (long long)X * Y;
    const size_t smem = (size_t)(2 * s.rows + s.dmax + 1) * sizeof(double);
    if (smem > kTableSmemMax) return ST_BAD_ARG;
    P.table_smem = smem > P.table_smem ? smem : P.table_smem;
    P.max_nx = X > P.max_nx ? X : P.max_nx;
    P.max_ny = Y > P.max_ny ? Y : P.max_ny;
  }
  P.nyw_count = (long long)P.nyw.size();
  return ST_OK;
}

// ---------------------------------------------------------------------------
// Weight table of one (period, row j): for window row r (latitude j1 = n1 + r)
// and column offset d (0..dmax)
//   a     = sin(dlat/2)^2 + sin(dlon/2)^2 cos(lat_j) cos(lat_j1)
//   delta = radius * 2 atan2(sqrt(a), sqrt(1 - a)) * km2deg
//   w     = exp(-delta^2 / (2 sigma^2))
// with dlat = (lat_j - lat_j1) deg2rad and dlon = (lon_d - lon_0) deg2rad,
// the terms of gps2dist_2 (utils.f90:1280-1294) and of :1220.  The per-row
// factors sin(dlat/2)^2 and cos(lat_j) cos(lat_j1) and the per-offset
// sin(dlon/2)^2 are evaluated once in shared memory.  Then one thread per
// window row writes the prefix sums P[r][k] = w[r][0] + ... + w[r][k], and
// one thread per clipping k the row's weight sums DL[k], DR[k].
// Grid (max_ny, nperiod); 128 threads.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_smooth_table(SmoothArgs A) {
  const SmoothPeriod P = A.per[blockIdx.y];
  const int j = blockIdx.x;
  if (j >= P.ny) return;
  extern __shared__ double sh[];
  const double* lons = A.lons + P.xoff;
  const double* lats = A.lats + P.yoff;
  const int nyw = A.nyw[P.woff + j];
  const int n1 = max(0, j - nyw), n2 = min(P.ny - 1, j + nyw), nr = n2 - n1 + 1;
  const int W = P.dmax + 1;
  double* s1s = sh;       // [nr]
  double* cc = sh + nr;   // [nr]
  double* s2s = sh + 2 * nr;  // [W]
  const double lat0 = lats[j];
  const double c0 = cos(lat0 * kDeg2Rad);
  for (int r = threadIdx.x; r < nr; r += blockDim.x) {
    const double lat1 = lats[n1 + r];
    const double s1 = sin((lat0 - lat1) * kDeg2Rad * 0.5);
    s1s[r] = s1 * s1;
    cc[r] = c0 * cos(lat1 * kDeg2Rad);
  }
  for (int d = threadIdx.x; d < W; d += blockDim.x) {
    const double s2 = sin((lons[d] - lons[0]) * kDeg2Rad * 0.5);
    s2s[d] = s2 * s2;
  }
  __syncthreads();
  double* wt = A.table + P.toff + (long long)j * smooth_row_doubles(P);
  double* pt = wt + (long long)P.rows * W;
  const double two_sigma_sq = 2.0 * (P.sigma * P.sigma);
  for (int e = threadIdx.x; e < nr * W; e += blockDim.x) {
    const int r = e / W, d = e - r * W;
    const double a = s1s[r] + s2s[d] * cc[r];
    const double delta = kRadius * (2.0 * atan2(sqrt(a), sqrt(1.0 - a))) * kKm2Deg;
    wt[e] = exp(-(delta * delta) / two_sigma_sq);
  }
  __syncthreads();
  for (int r = threadIdx.x; r < nr; r += blockDim.x) {
    double s = 0.0;
    for (int d = 0; d < W; ++d) {
      s += wt[r * W + d];
      pt[r * W + d] = s;
    }
  }
  __syncthreads();
  double* dl = pt + (long long)P.rows * W;
  double* dr = dl + W;
  for (int k = threadIdx.x; k < W; k += blockDim.x) {
    double l = 0.0, r = 0.0;
    for (int q = 0; q < nr; ++q) {
      l += pt[q * W + k] - wt[q * W];
      r += pt[q * W + k];
    }
    dl[k] = l;
    dr[k] = r;
  }
}

// ---------------------------------------------------------------------------
// Apply: one thread per output node, nodes numbered period by period and row
// by row (no idle lanes at row ends).  Over the window rows in order,
//   num += w[r][|d|] * data(i + d, n1 + r)   for d = -kl .. kr (ascending column)
// with kl = min(nxw, i), kr = min(nxw, nx-1-i) (the clamped window of
// :1216-1217); out = num / (DL[kl] + DR[kr]) (:1222-1223).  Lanes of a warp
// hold adjacent columns: the table reads are warp-uniform within a row, the
// data reads coalesced.  Grid ceil(nodes / 128); 128 threads.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_smooth_apply(SmoothArgs A) {
  const long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (n >= A.nodes) return;
  int lo = 0, hi = A.nperiod - 1;  // period of node n
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&A.per[mid].node0) <= n) lo = mid;
    else hi = mid - 1;
  }
  const SmoothPeriod& P = A.per[lo];
  const int nx = __ldg(&P.nx), nxw = __ldg(&P.nxw), W = __ldg(&P.dmax) + 1;
  const int rows = __ldg(&P.rows), ny = __ldg(&P.ny);
  const int k = (int)(n - __ldg(&P.node0));
  const int j = k / nx, i = k - j * nx;
  const int nyw = __ldg(A.nyw + __ldg(&P.woff) + j);
  const int n1 = max(0, j - nyw), n2 = min(ny - 1, j + nyw);
  const int kl = min(nxw, i), kr = min(nxw, nx - 1 - i);
  const double* wt = A.table + __ldg(&P.toff) + (long long)j * (2LL * (rows + 1) * W);
  const double* dl = wt + 2LL * rows * W;
  const double den = __ldg(dl + kl) + __ldg(dl + W + kr);
  const double* col = A.data + __ldg(&P.doff) + i;
  double num = 0.0;
  for (int r = 0; r <= n2 - n1; ++r) {
    const double* w = wt + r * W;
    const double* x = col + (long long)(n1 + r) * nx;
#pragma unroll 4
    for (int d = kl; d >= 1; --d) num = fma(__ldg(w + d), __ldg(x - d), num);
#pragma unroll 4
    for (int d = 0; d <= kr; ++d) num = fma(__ldg(w + d), __ldg(x + d), num);
  }
  A.out[__ldg(&P.goff) + k] = num / den;
}

void launch_smooth_table(const SmoothArgs& A, const SmoothPlan& plan, cudaStream_t st) {
  if (A.nperiod <= 0 || plan.max_ny <= 0) return;
  if (plan.table_smem > 48 * 1024)
    cudaFuncSetAttribute(k_smooth_table, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)plan.table_smem);
  k_smooth_table<<<dim3(plan.max_ny, A.nperiod), 128, plan.table_smem, st>>>(A);
}

void launch_smooth_apply(const SmoothArgs& A, const SmoothPlan& plan, cudaStream_t st) {
  if (A.nperiod <= 0 || plan.nodes <= 0) return;
  k_smooth_apply<<<(unsigned)((plan.nodes + 127) / 128), 128, 0, st>>>(A);
}

}  // namespace sgb
