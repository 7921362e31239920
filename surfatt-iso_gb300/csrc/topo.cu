// topo.cu -- the surface metric of SurfATT's curved-surface eikonal from a
// topography grid (get_topo, src/grid.f90:117-145): per period the
// topography smoothed by gaussian_smooth_geo_2 with that period's sigma
// (src/topo.f90:74-81, the smoothing kernels of smooth.cu, every period in
// one launch), its spherical gradient (gradient_2_geo,
// src/shared/utils.f90:1118-1160), the metric a, b, c and the dip angle
// (calc_dip_angle, src/topo.f90:119-127).
#include <cmath>
#include <vector>

#include "../../include/surfatt_gb300.h"
#include "common.cuh"
#include "host_buf.cuh"
#include "smooth.cuh"

using namespace sgb;

namespace {

struct TopoArgs {
  int nx, ny, P;
  const double* sm;    // smoothed topography: P fields of nx*ny, period by period
  const double* lon;   // (nx) degrees
  const double* lat;   // (ny)
  const double* cosd;  // (ny) cosd(lat), evaluated on the host
  double *m11, *m22, *m12, *angle;  // (P, nx, ny), period fastest; any may be null
};

// One thread per (period, node), the period fastest (coalesced stores in
// the reference's layout).  gradient_2_geo: dx(i) = R*(lon(i)-lon(i-1))*
// deg2rad*cosd(lat(j)), central differences (gfx+gbx)/(2 dx) inside, one-
// sided at the edges with dx of the second / last node; the same in y
// without the cosine.  Then a = (1+fy^2)/(1+fx^2+fy^2),
// b = (1+fx^2)/(...), c = fx*fy/(...), m11 = a, m22 = b, m12 = -c
// (src/grid.f90:121-123, :142-145) and atand(sqrt(fx^2+fy^2)).  All but the
// arctangent are explicitly rounded IEEE operations, as written.
__global__ void __launch_bounds__(128) k_topo_metric(TopoArgs A) {
  const long long N = (long long)A.nx * A.ny;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= N * A.P) return;
  const int p = (int)(t % A.P);
  const long long e = t / A.P;
  const int nx = A.nx, ny = A.ny;
  const int i = (int)(e % nx), j = (int)(e / nx);
  const double* f = A.sm + (long long)p * N;
  const double R = 6371.0, d2r = PI_S / 180.0;
  const double cj = __ldg(A.cosd + j);
  auto DX = [&](int ix) {
    return __dmul_rn(__dmul_rn(__dmul_rn(R, __dsub_rn(__ldg(A.lon + ix), __ldg(A.lon + ix - 1))),
                               d2r),
                     cj);
  };
  auto DY = [&](int iy) {
    return __dmul_rn(__dmul_rn(R, __dsub_rn(__ldg(A.lat + iy), __ldg(A.lat + iy - 1))), d2r);
  };
  const double fc = __ldg(f + e);
  double x, y;
  if (i == 0) x = __ddiv_rn(__dsub_rn(__ldg(f + e + 1), fc), DX(1));
  else if (i == nx - 1) x = __ddiv_rn(__dsub_rn(fc, __ldg(f + e - 1)), DX(nx - 1));
  else
    x = __ddiv_rn(__dadd_rn(__dsub_rn(fc, __ldg(f + e - 1)), __dsub_rn(__ldg(f + e + 1), fc)),
                  __dmul_rn(2.0, DX(i)));
  if (j == 0) y = __ddiv_rn(__dsub_rn(__ldg(f + e + nx), fc), DY(1));
  else if (j == ny - 1) y = __ddiv_rn(__dsub_rn(fc, __ldg(f + e - nx)), DY(ny - 1));
  else
    y = __ddiv_rn(__dadd_rn(__dsub_rn(fc, __ldg(f + e - nx)), __dsub_rn(__ldg(f + e + nx), fc)),
                  __dmul_rn(2.0, DY(j)));
  const double xx = __dmul_rn(x, x), yy = __dmul_rn(y, y);
  const double den = __dadd_rn(__dadd_rn(1.0, xx), yy);
  if (A.m11) A.m11[t] = __ddiv_rn(__dadd_rn(1.0, yy), den);
  if (A.m22) A.m22[t] = __ddiv_rn(__dadd_rn(1.0, xx), den);
  if (A.m12) A.m12[t] = -__ddiv_rn(__dmul_rn(x, y), den);
  if (A.angle) A.angle[t] = atan(__dsqrt_rn(__dadd_rn(xx, yy))) * (180.0 / 3.14159265358979323846);
}

struct TopoCtx {
  bool init = false;
  cudaStream_t st = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool timed = false;
  DBuf topo, lon, lat, cosd, nyw, per, tab, sm, m11, m22, m12, ang;
  ~TopoCtx() {
    if (!init) return;
    for (DBuf* d : {&topo, &lon, &lat, &cosd, &nyw, &per, &tab, &sm, &m11, &m22, &m12, &ang})
      d->release();
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    cudaStreamDestroy(st);
  }
  int setup() {
    if (init) return SURFATT_OK;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ev0) != cudaSuccess || cudaEventCreate(&ev1) != cudaSuccess) {
      // a partial setup is undone, so that the next call starts afresh
      if (ev0) cudaEventDestroy(ev0);
      if (ev1) cudaEventDestroy(ev1);
      if (st) cudaStreamDestroy(st);
      ev0 = ev1 = nullptr;
      st = nullptr;
      cudaGetLastError();
      return SURFATT_CUDA_ERROR;
    }
    init = true;
    return SURFATT_OK;
  }
};

thread_local TopoCtx g_tc;

int up(TopoCtx& c, DBuf& b, const void* src, size_t bytes) {
  if (b.ensure(bytes ? bytes : 8)) return SURFATT_OOM;
  if (src && bytes) CK(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, c.st));
  return SURFATT_OK;
}

}  // namespace

extern "C" {

surfatt_status_t surfatt_topo_sigma(int nperiod, const double* phase_vel, const double* periods,
                                    double wavelen_factor, double* sigma) {
  if (nperiod < 0 || !phase_vel || !periods || !sigma) return SURFATT_BAD_ARG;
  const double km2deg = 1.0 / (6371.0 * PI_S / 180.0);
  for (int p = 0; p < nperiod; ++p)  // src/grid.f90:117
    sigma[p] = phase_vel[p] * periods[p] * wavelen_factor * km2deg / (2.0 * PI_S);
  return SURFATT_OK;
}

surfatt_status_t surfatt_topo_metric(const double* topo, int nx, int ny, const double* lon,
                                     const double* lat, int nperiod, const double* sigma,
                                     double* m11, double* m22, double* m12, double* topo_angle) {
  if (!topo || !lon || !lat || !sigma || nperiod < 1) return SURFATT_BAD_ARG;
  const long long N = (long long)nx * ny;
  std::vector<int> vnx(nperiod, nx), vny(nperiod, ny);
  std::vector<long long> goff(nperiod), zero(nperiod, 0);
  for (int p = 0; p < nperiod; ++p) goff[p] = p * N;
  SmoothPlan plan;
  if (smooth_plan(nperiod, vnx.data(), vny.data(), goff.data(), zero.data(), zero.data(),
                  zero.data(), lon, lat, sigma, &plan) != ST_OK)
    return SURFATT_BAD_ARG;
  TopoCtx& c = g_tc;
  int r = c.setup();
  if (r) return (surfatt_status_t)r;
  std::vector<double> cosd(ny);
  for (int j = 0; j < ny; ++j) cosd[j] = std::cos(lat[j] * (3.14159265358979323846 / 180.0));
  const size_t d = sizeof(double), PN = (size_t)nperiod * N;
  r = up(c, c.topo, topo, N * d);
  r = r ? r : up(c, c.lon, lon, nx * d);
  r = r ? r : up(c, c.lat, lat, ny * d);
  r = r ? r : up(c, c.cosd, cosd.data(), ny * d);
  r = r ? r : up(c, c.nyw, plan.nyw.data(), plan.nyw_count * sizeof(int));
  r = r ? r : up(c, c.per, plan.per.data(), plan.per.size() * sizeof(SmoothPeriod));
  r = r ? r : up(c, c.tab, nullptr, plan.table_doubles * d);
  r = r ? r : up(c, c.sm, nullptr, PN * d);
  r = r ? r : up(c, c.m11, nullptr, m11 ? PN * d : 0);
  r = r ? r : up(c, c.m22, nullptr, m22 ? PN * d : 0);
  r = r ? r : up(c, c.m12, nullptr, m12 ? PN * d : 0);
  r = r ? r : up(c, c.ang, nullptr, topo_angle ? PN * d : 0);
  if (r) return (surfatt_status_t)r;
  SmoothArgs S{c.per.as<SmoothPeriod>(), nperiod, c.lon.as<double>(), c.lat.as<double>(),
               c.nyw.as<int>(), c.topo.as<double>(), c.sm.as<double>(), c.tab.as<double>(),
               plan.nodes};
  TopoArgs T{nx,
             ny,
             nperiod,
             c.sm.as<double>(),
             c.lon.as<double>(),
             c.lat.as<double>(),
             c.cosd.as<double>(),
             m11 ? c.m11.as<double>() : nullptr,
             m22 ? c.m22.as<double>() : nullptr,
             m12 ? c.m12.as<double>() : nullptr,
             topo_angle ? c.ang.as<double>() : nullptr};
  CK(cudaEventRecord(c.ev0, c.st));
  launch_smooth_table(S, plan, c.st);
  launch_smooth_apply(S, plan, c.st);
  k_topo_metric<<<(unsigned)((PN + 127) / 128), 128, 0, c.st>>>(T);
  CK(cudaGetLastError());
  CK(cudaEventRecord(c.ev1, c.st));
  c.timed = true;
  if (m11) CK(cudaMemcpyAsync(m11, c.m11.p, PN * d, cudaMemcpyDeviceToHost, c.st));
  if (m22) CK(cudaMemcpyAsync(m22, c.m22.p, PN * d, cudaMemcpyDeviceToHost, c.st));
  if (m12) CK(cudaMemcpyAsync(m12, c.m12.p, PN * d, cudaMemcpyDeviceToHost, c.st));
  if (topo_angle) CK(cudaMemcpyAsync(topo_angle, c.ang.p, PN * d, cudaMemcpyDeviceToHost, c.st));
  CK(cudaStreamSynchronize(c.st));
  return SURFATT_OK;
}

surfatt_status_t surfatt_topo_metric_timing(double* kernel_ms, int* launches) {
  TopoCtx& c = g_tc;
  if (!c.timed) return SURFATT_BAD_ARG;
  CK(cudaEventSynchronize(c.ev1));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
  if (kernel_ms) *kernel_ms = ms;
  if (launches) *launches = 3;
  return SURFATT_OK;
}

}  // extern "C"
