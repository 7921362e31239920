// common.cuh -- shared device definitions of the SurfATT GB300 kernels.
//
// Arrays follow the reference's Fortran layout: a field of one period is
// (nx, ny) column-major, element (i, j) at [i + nx*j], x (longitude) fastest.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sgb {

// Literal constants of src/eikon_solver_2d.f90 as gfortran evaluates them:
// default-real literals are single precision (no `implicit none`, no
// -fdefault-real-8 in CMakeLists.txt:24-29).
constexpr double PI_S = (double)3.14159265358979323846f;  // :785, :1297
constexpr double R_EARTH = 6371.0;                         // :777, :1296
constexpr double TOL_UW = (double)1e-4f;                   // :775
constexpr double TOL_JSE = (double)1e-9f;                  // :1294
constexpr double TOL_WENO = (double)1e-6f;                 // :353, :559
constexpr double EPS14 = (double)1e-14f;                   // :775, :1294
constexpr int MAXITER_UW = 2000;                           // :774
constexpr int MAXITER_JSE = 1000;                          // :1293
constexpr int MAXITER_WENO = 1000;                         // :352, :558

enum Status : int {
  ST_OK = 0,
  ST_SOURCE_ON_BOUNDARY = 1,
  ST_BAD_ARG = 2,
  ST_NOT_CONVERGED = 3,
  ST_OOM = 4,
  ST_CUDA_ERROR = 5,
  ST_TIMEOUT = 6
};

// Per-period fields in sweep units, shared by every solve of the period.
// For lon/lat grids (xs, ys) are radians and a, b, c carry the spherical
// metric of :817-821; for Cartesian grids they are the caller's values.
struct PeriodDev {
  int nx, ny;
  int lonlat;
  double dx, dy;                       // sweep units
  const double* xs;                    // (nx) node coordinates, sweep units
  const double* ys;                    // (ny)
  const double* xdeg;                  // (nx) caller's coordinates (interp2, mask)
  const double* ydeg;                  // (ny)
  const double* cosy;                  // (ny) cos(ys), lon/lat only
  const double* siny;                  // (ny) sin(ys), lon/lat only
  const double* a;                     // (N)
  const double* b;
  const double* c;
  const double* fun;                   // slowness 1/vel
  const double* f2;                    // fun**2
  const double* disx;                  // sqrt(fun**2*(b/(a*b-c**2)))  (:1014)
  const double* disy;                  // sqrt(fun**2*(a/(a*b-c**2)))  (:1055)
  const double* svel;                  // phase velocity (kernel division)
  long long goff;                      // cell offset of the period in packed arrays
  // FP32 copies for the FP32-factored sweeps (null when not prepared):
  // f32 + m*N, m = 0..5: a, b, c, fun**2, disx, disy
  const float* f32;
  // 1/svel**2 and 1/svel**3 (isv, isv + N) for the FP32 path's kernel slots
  const double* isv;
  // per-cell FP32 record of 32 bytes: p4a[2k] = {a, b, c, fun**2} and
  // p4b[2k] = p4a[2k + 1] = {disx, disy, 1/svel**2, 1/svel**3} (p4b = p4a + 1)
  const float4* p4a;
  const float4* p4b;
};

// Source/receiver cell and REAL(4) bilinear weights:
//   idx0 = floor((x0-xx(1))/dx+1);  r1 = min(1.0,(x0-xx(idx0))/dx)   (:828-829)
// `limit` = largest admissible 0-based cell + 1.  Returns -1 when outside.
__host__ __device__ inline int locate_cell(const double* xx, int limit, double dx, double x0,
                                           float* r) {
  double f = floor((x0 - xx[0]) / dx + 1.0);
  if (!(f >= 1.0) || f > (double)limit) return -1;
  int i = (int)f - 1;
  double q = (x0 - xx[i]) / dx;
  *r = (float)(q < 1.0 ? q : 1.0);
  return i;
}

// Approximate reciprocal and square root of the FP32 sweeps (hardware MUFU,
// about 2 ulp, no special-case branches): the update adds their products to
// tau_X as a small increment, so this error stays far below FP32 resolution
// of tau.  sqrt of a non-positive argument returns 0 (its root is rejected by
// the caller's D >= 0 test).
__device__ __forceinline__ float frcp_fast(float x) { return __fdividef(1.0f, x); }
__device__ __forceinline__ float fsqrt_fast(float x) { return x > 0.f ? x * rsqrtf(x) : 0.f; }

// Block-wide reductions (blockDim.x a multiple of 32, <= 1024).
__device__ inline double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ inline double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Sum and max over the block; every thread receives both results.
// `red` must hold 2*32 doubles of shared memory.
__device__ inline void block_sum_max(double& s, double& m, double* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  s = warp_sum(s);
  m = warp_max(m);
  __syncthreads();
  if (lane == 0) {
    red[wid] = s;
    red[32 + wid] = m;
  }
  __syncthreads();
  double ts = 0.0, tm = 0.0;
  for (int w = 0; w < nw; ++w) {  // fixed order: deterministic
    ts += red[w];
    tm = fmax(tm, red[32 + w]);
  }
  s = ts;
  m = tm;
  __syncthreads();
}

// Diagonal walk of one sweep ordering: logical coordinates (u, v) with
// u = xdir>0 ? i : nx-1-i, v = ydir>0 ? j : ny-1-j over the rectangle
// [ilo, ihi] x [jlo, jhi] (inclusive); cells with u+v = d are independent,
// and visiting d = 0, 1, ... reproduces the in-place Gauss-Seidel order of
// the reference's nested x-outer / y-inner loops exactly (every stencil only
// reaches along the axes).
struct SweepGeom {
  int ilo, ihi, jlo, jhi, xdir, ydir;
  __device__ int nu() const { return ihi - ilo + 1; }
  __device__ int nv() const { return jhi - jlo + 1; }
  __device__ int ndiag() const { return nu() + nv() - 1; }
  __device__ int vmin(int d) const { return d - (nu() - 1) > 0 ? d - (nu() - 1) : 0; }
  __device__ int vmax(int d) const { return d < nv() - 1 ? d : nv() - 1; }
  __device__ void cell(int d, int v, int& i, int& j) const {
    int u = d - v;
    i = xdir > 0 ? ilo + u : ihi - u;
    j = ydir > 0 ? jlo + v : jhi - v;
  }
};

// Sweep orderings of the reference: forward UW (:884-902) and the
// nint-bounded adjoint / WENO loops (:1386-1390) both visit
// (x+,y+), (x+,y-), (x-,y+), (x-,y-) in that order.
__device__ inline void sweep_dirs(int s, int& xdir, int& ydir) {
  xdir = s < 2 ? 1 : -1;
  ydir = (s == 0 || s == 2) ? 1 : -1;
}

}  // namespace sgb
