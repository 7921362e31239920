// noalloc.cu -- a forward lon/lat eikonal solve that allocates no memory.
//
// Who needs it: callers that must not allocate device memory when they call
// the solver -- for example a host framework whose own memory pool owns the
// GPU's HBM (an extra cudaMalloc would bypass its budget), or a loop that
// cannot afford cudaMalloc/cudaFree (cudaFree synchronises the whole device
// and stalls every other stream).  The ordinary entry point
// fsm_uw_ps_lonlat_2d_ allocates its scratch on first use and copies host
// arrays; this one takes device arrays and a stream and uses a fixed scratch
// area compiled into the library instead.
//
// The scratch is the file-scope array g_noalloc_scratch below: every GPU that
// loads the library holds it (NOALLOC_SCRATCH_BYTES, about 4.8 MB) until the
// process exits.  Host code cannot use the array's name as a device address,
// so the first call on each device looks the address up with
// cudaGetSymbolAddress (with that device current) and caches it; make that
// first call before any stream capture.  The cached address belongs to the
// device's context: after cudaDeviceReset (which destroys that context and
// the array with it) the entry point must not be called again in the same
// process.  All calls share the one array,
// which keeps whatever the last call left there; a call reads only scratch
// words it has written itself earlier in the same call (nothing needs to
// start at zero), so results do not depend on the previous call -- but two
// calls whose kernels overlap on the GPU (different streams with no ordering
// between them) race on the array and corrupt each other.
#include <cstdio>
#include <mutex>

#include "../../include/surfatt_gb300.h"
#include "solver_fp64.cuh"

namespace sgb {
namespace {

constexpr long long NOALLOC_MAX_CELLS = 16384;  // nx*ny limit (e.g. 128 x 128)
constexpr int NOALLOC_MAX_AXIS = 2048;          // nx, ny limit
// forward workspace (tau, tau_old, T0 + hoisted constants) + per-grid fields
// (a, b, c, fun, f2, disx, disy) + axis arrays (xs, ys, cosy, siny)
constexpr long long NOALLOC_FIELDS = 3 + (long long)KC_COUNT + 7;
constexpr long long NOALLOC_SCRATCH_DOUBLES =
    NOALLOC_FIELDS * NOALLOC_MAX_CELLS + 4LL * NOALLOC_MAX_AXIS;
constexpr long long NOALLOC_SCRATCH_BYTES = NOALLOC_SCRATCH_DOUBLES * 8;

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
double* g_addr[MAX_DEVICES] = {nullptr};

// One block: per-grid precompute (as k_prep) into the scratch, then the same
// forward setup and sweeps as the drop-in's single-solve kernel.
__global__ void __launch_bounds__(256) k_uw_noalloc(const double* xdeg, const double* ydeg,
                                                    int nx, int ny, const double* spha,
                                                    const double* sphb, const double* sphc,
                                                    const double* fun_in, double x0, double y0,
                                                    double* scratch, double* T, int* si) {
  __shared__ SolveShared sh;
  const size_t N = (size_t)nx * ny;
  double* p = scratch;
  FwdWs W;
  W.tau = p; p += N;
  W.tau_old = p; p += N;
  W.T0 = p; p += N;
  W.K = p; p += (size_t)KC_COUNT * N;
  double *a = p, *b = p + N, *c = p + 2 * N, *fun = p + 3 * N, *f2 = p + 4 * N,
         *disx = p + 5 * N, *disy = p + 6 * N;
  p += 7 * N;
  double *xs = p, *ys = p + nx, *cosy = p + nx + ny, *siny = p + nx + 2 * ny;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) xs[i] = xdeg[i] / 180.0 * PI_S;
  for (int j = threadIdx.x; j < ny; j += blockDim.x) {
    const double y = ydeg[j] / 180.0 * PI_S;
    ys[j] = y;
    cosy[j] = cos(y);
    siny[j] = sin(y);
  }
  for (size_t k = threadIdx.x; k < N; k += blockDim.x) {
    const int j = (int)(k / nx);
    const double y = ydeg[j] / 180.0 * PI_S;
    const double cy = cos(y);
    const double aa = spha[k] / (R_EARTH * R_EARTH * (cy * cy));
    const double bb = sphb[k] / (R_EARTH * R_EARTH);
    const double cc = sphc[k] / (R_EARTH * R_EARTH * cy);
    const double f = fun_in[k];
    a[k] = aa;
    b[k] = bb;
    c[k] = cc;
    fun[k] = f;
    f2[k] = f * f;
    disx[k] = sqrt(f * f * (bb / (aa * bb - cc * cc)));
    disy[k] = sqrt(f * f * (aa / (aa * bb - cc * cc)));
  }
  __syncthreads();
  PeriodDev P;
  P.nx = nx;
  P.ny = ny;
  P.lonlat = 1;
  P.dx = xs[1] - xs[0];
  P.dy = ys[1] - ys[0];
  P.xs = xs;
  P.ys = ys;
  P.xdeg = xdeg;
  P.ydeg = ydeg;
  P.cosy = cosy;
  P.siny = siny;
  P.a = a;
  P.b = b;
  P.c = c;
  P.fun = fun;
  P.f2 = f2;
  P.disx = disx;
  P.disy = disy;
  P.svel = nullptr;
  P.goff = 0;
  P.f32 = nullptr;
  P.isv = nullptr;
  P.p4a = nullptr;
  P.p4b = nullptr;
  fwd_setup(P, x0, y0, 1.0, 1.0, 10.0, W, true, sh);
  if (sh.status != ST_OK) {
    if (threadIdx.x == 0) { si[0] = sh.status; si[1] = 0; }
    return;
  }
  uw_sweeps(P, W, sh, MAXITER_UW);
  for (size_t k = threadIdx.x; k < N; k += blockDim.x) T[k] = W.tau[k] * W.T0[k];
  if (threadIdx.x == 0) { si[0] = sh.status; si[1] = sh.iters; }
}

}  // namespace
}  // namespace sgb

extern "C" surfatt_status_t surfatt_uw_lonlat_solve_noalloc(
    const double* xx_deg, const double* yy_deg, int nx, int ny, const double* spha,
    const double* sphb, const double* sphc, const double* fun, double x0_deg, double y0_deg,
    double* T, int* status_iters, void* stream) {
  using namespace sgb;
  if (!xx_deg || !yy_deg || !spha || !sphb || !sphc || !fun || !T || !status_iters)
    return SURFATT_BAD_ARG;
  if (nx < 2 || ny < 2 || nx > NOALLOC_MAX_AXIS || ny > NOALLOC_MAX_AXIS ||
      (long long)nx * ny > NOALLOC_MAX_CELLS) {
    std::fprintf(stderr,
                 "surfatt_uw_lonlat_solve_noalloc: grid %d x %d exceeds the fixed scratch "
                 "(at most %lld cells, %d per axis)\n",
                 nx, ny, NOALLOC_MAX_CELLS, NOALLOC_MAX_AXIS);
    return SURFATT_BAD_ARG;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return SURFATT_CUDA_ERROR;
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
      void* ptr = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess || !ptr) {
        std::fprintf(stderr, "surfatt_uw_lonlat_solve_noalloc: cudaGetSymbolAddress failed: %s\n",
                     cudaGetErrorString(e));
        return SURFATT_CUDA_ERROR;
      }
      g_addr[dev] = static_cast<double*>(ptr);
    }
    scratch = g_addr[dev];
  }
  double x0 = x0_deg / 180.0 * PI_S, y0 = y0_deg / 180.0 * PI_S;
  // cudaLaunchKernel returns this launch's own error: an error that earlier,
  // unrelated work left pending on the thread is neither reported as this
  // call's failure nor cleared from under its owner.
  void* args[] = {&xx_deg, &yy_deg, &nx, &ny, &spha, &sphb, &sphc, &fun,
                  &x0, &y0, &scratch, &T, &status_iters};
  const cudaError_t e = cudaLaunchKernel(reinterpret_cast<const void*>(&k_uw_noalloc), dim3(1),
                                         dim3(256), args, 0, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? SURFATT_OK : SURFATT_CUDA_ERROR;
}
