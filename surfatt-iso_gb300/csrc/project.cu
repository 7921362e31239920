// project.cu -- kernel combination (combine_kernels) and multigrid
// projection (inv_grid_iso / inv2fwd_iso, post_processing_for_kernel) of
// SurfATT's 3-D inversion on the GPU.  See project.cuh for the ordering and
// tie-resolution rules that make the results the reference's bit for bit.
#include <cmath>

#include "common.cuh"
#include "project.cuh"

namespace sgb {

namespace {

// One axis of locate_within_cube (src/eikon_solver_2d.f90:1476-1490): the
// walking search from cell `start` (1-based).  Returns the 0-based cell, or
// -1 when the walk leaves the grid; *w the interpolation weight.
int walk(double x, int n, const double* v, int start, double* w) {
  int i1 = start;
  while (i1 > 0 && i1 < n) {
    const int i2 = i1 + 1;
    if (x < v[i1 - 1]) {
      --i1;
    } else if (x <= v[i2 - 1]) {
      *w = (x - v[i1 - 1]) / (v[i2 - 1] - v[i1 - 1]);
      return i1 - 1;
    } else {
      ++i1;
    }
  }
  *w = 0.0;
  return -1;
}

void build_axis(const double* coords, int n, const double* inv, int ninv, int nset,
                ProjAxis* A) {
  A->n = n;
  A->ninv = ninv;
  A->cell.assign((size_t)nset * 2 * n, -1);
  A->w.assign((size_t)nset * 2 * n, 0.0);
  A->rng.assign((size_t)nset * ninv, make_int2(1, 0));
  for (int s = 0; s < nset; ++s) {
    const double* v = inv + (size_t)ninv * s;
    for (int i = 0; i < n; ++i) {
      double w = 0;
      const int lo = walk(coords[i], ninv, v, 1, &w);
      A->cell[(size_t)(2 * s) * n + i] = lo;
      A->w[(size_t)(2 * s) * n + i] = w;
      const int up = walk(coords[i], ninv, v, ninv - 1, &w);
      A->cell[(size_t)(2 * s + 1) * n + i] = up;
      A->w[(size_t)(2 * s + 1) * n + i] = w;
      if (i < 1 || i > n - 2) continue;  // inv_grid_iso visits interior nodes
      for (int c : {lo, up}) {
        if (c < 0) continue;
        for (int a : {c, c + 1}) {  // corners of cell c
          int2& r = A->rng[(size_t)ninv * s + a];
          if (r.x > r.y) {
            r.x = r.y = i;
          } else {
            r.x = i < r.x ? i : r.x;
            r.y = i > r.y ? i : r.y;
          }
        }
      }
    }
  }
}

bool found(const ProjAxis& A, int s, int i) { return A.cell[(size_t)(2 * s) * A.n + i] >= 0; }

// First node of a projection's loops (sets, then j, i, k) that is not
// located; lo = 1 for inv_grid_iso (interior nodes), 0 for inv2fwd_iso.
bool first_bad(const ProjPlan& P, int lo, const double* vx, const double* vy, const double* vz,
               double* xyz) {
  for (int s = 0; s < P.nset; ++s)
    for (int j = lo; j <= P.ny - 1 - lo; ++j)
      for (int i = lo; i <= P.nx - 1 - lo; ++i)
        for (int k = lo; k <= P.nz - 1 - lo; ++k)
          if (!(found(P.ax[0], s, i) && found(P.ax[1], s, j) && found(P.ax[2], s, k))) {
            xyz[0] = vx[i];
            xyz[1] = vy[j];
            xyz[2] = vz[k];
            return true;
          }
  return false;
}

}  // namespace

int proj_plan(const double* xinv, const double* yinv, const double* zinv, int nxinv, int nyinv,
              int nzinv, int nset, const double* vx, const double* vy, const double* vz, int nx,
              int ny, int nz, int need, ProjPlan* plan) {
  ProjPlan& P = *plan;
  P = ProjPlan();
  if (nx < 2 || ny < 2 || nz < 2 || nxinv < 2 || nyinv < 2 || nzinv < 2 || nset < 1 ||
      nxinv > 1024 || nyinv > 1024 || nzinv > 1024)  // cells are packed in 10 bits per axis
    return ST_BAD_ARG;
  P.nx = nx;
  P.ny = ny;
  P.nz = nz;
  P.nset = nset;
  P.dx = vx[1] - vx[0];
  P.dy = vy[1] - vy[0];
  P.dz = vz[1] - vz[0];
  build_axis(vx, nx, xinv, nxinv, nset, &P.ax[0]);
  build_axis(vy, ny, yinv, nyinv, nset, &P.ax[1]);
  build_axis(vz, nz, zinv, nzinv, nset, &P.ax[2]);
  if ((need & 1) && first_bad(P, 1, vx, vy, vz, P.bad_xyz)) P.bad = 1;
  else if ((need & 2) && first_bad(P, 0, vx, vy, vz, P.bad_xyz)) P.bad = 2;
  return P.bad ? 7 : ST_OK;
}

void proj_pack(const ProjPlan& plan, ProjTables* t) {
  t->cells.clear();
  t->w.clear();
  t->rng.clear();
  for (int a = 0; a < 3; ++a) {
    const ProjAxis& A = plan.ax[a];
    t->cell_off[a] = (long long)t->cells.size();
    t->w_off[a] = (long long)t->w.size();
    t->rng_off[a] = (long long)t->rng.size();
    t->cells.insert(t->cells.end(), A.cell.begin(), A.cell.end());
    t->w.insert(t->w.end(), A.w.begin(), A.w.end());
    t->rng.insert(t->rng.end(), A.rng.begin(), A.rng.end());
  }
}

ProjDev proj_dev(const ProjPlan& plan, const ProjTables& t, const int* d_cells, const double* d_w,
                 const int2* d_rng) {
  ProjDev D;
  D.nx = plan.nx;
  D.ny = plan.ny;
  D.nz = plan.nz;
  D.nset = plan.nset;
  D.dx = plan.dx;
  D.dy = plan.dy;
  D.dz = plan.dz;
  for (int a = 0; a < 3; ++a) {
    D.ninv[a] = plan.ax[a].ninv;
    D.cell[a] = d_cells + t.cell_off[a];
    D.w[a] = d_w + t.w_off[a];
    D.rng[a] = d_rng + t.rng_off[a];
  }
  return D;
}

// ---------------------------------------------------------------------------
// combine_kernels (src/acqui.f90:196-245): one thread per model node; the
// sum over periods in the reference's order, each term associated as
// written.  dalpha_dbeta / drho_dalpha (src/shared/utils.f90:99-145) with
// their default-real coefficients (integer * literal folded in single
// precision) and x**2 = x*x, x**3 = (x*x)*x, x**4 = (x*x)*(x*x).
// ---------------------------------------------------------------------------
struct CombineArgs {
  int P, nx, ny, nz, rho_scaling;
  const double *adj_s, *adj_d, *svs, *svp, *srho, *vs, *vp;
  double *ker, *kd;
};

__device__ __forceinline__ double dalpha_dbeta(double vs) {
  const double c0 = (double)2.0947f, c1 = (double)(2 * 0.8206f);
  const double c2 = (double)(3 * 0.2683f), c3 = (double)(4 * 0.0251f);
  const double v2 = __dmul_rn(vs, vs), v3 = __dmul_rn(v2, vs);
  double r = __dsub_rn(c0, __dmul_rn(c1, vs));
  r = __dadd_rn(r, __dmul_rn(c2, v2));
  return __dsub_rn(r, __dmul_rn(c3, v3));
}

__device__ __forceinline__ double drho_dalpha(double vp) {
  const double c0 = (double)1.6612f, c1 = (double)(2 * 0.4721f);
  const double c2 = (double)(3 * 0.0671f), c3 = (double)(4 * 0.0043f);
  const double c4 = (double)(5 * 0.000106f);
  const double v2 = __dmul_rn(vp, vp), v3 = __dmul_rn(v2, vp), v4 = __dmul_rn(v2, v2);
  double r = __dsub_rn(c0, __dmul_rn(c1, vp));
  r = __dadd_rn(r, __dmul_rn(c2, v2));
  r = __dsub_rn(r, __dmul_rn(c3, v3));
  return __dadd_rn(r, __dmul_rn(c4, v4));
}

template <bool ABR>
__global__ void __launch_bounds__(128) k_combine(CombineArgs A) {
  const size_t N2 = (size_t)A.nx * A.ny, N3 = N2 * A.nz;
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= N3) return;
  const size_t e2 = e % N2;
  const int P = A.P;
  const double* as = A.adj_s + (size_t)P * e2;
  const double* ad = A.adj_d + (size_t)P * e2;
  const double* svs = A.svs + (size_t)P * e;
  const double* svp = A.svp + (size_t)P * e;
  const double* srho = A.srho + (size_t)P * e;
  if (ABR) {
    double k0 = 0.0, k1 = 0.0, k2 = 0.0, d0 = 0.0, d1 = 0.0, d2 = 0.0;
    for (int ip = 0; ip < P; ++ip) {
      const double a = __ldg(as + ip), b = __ldg(ad + ip);
      const double s0 = __ldg(svs + ip), s1 = __ldg(svp + ip);
      k0 = __dsub_rn(k0, __dmul_rn(a, s0));
      d0 = __dsub_rn(d0, __dmul_rn(b, s0));
      k1 = __dsub_rn(k1, __dmul_rn(a, s1));
      d1 = __dsub_rn(d1, __dmul_rn(b, s1));
      if (!A.rho_scaling) {
        const double s2 = __ldg(srho + ip);
        k2 = __dsub_rn(k2, __dmul_rn(a, s2));
        d2 = __dsub_rn(d2, __dmul_rn(b, s2));
      }
    }
    if (A.rho_scaling) {  // :222-225, rho_scaling = 0.33 (shared_par.f90:16)
      k2 = __dmul_rn((double)0.33f, k0);
      d2 = d0;
    }
    A.ker[3 * e] = k0;
    A.ker[3 * e + 1] = k1;
    A.ker[3 * e + 2] = k2;
    A.kd[3 * e] = d0;
    A.kd[3 * e + 1] = d1;
    A.kd[3 * e + 2] = d2;
  } else {
    const double dab = dalpha_dbeta(__ldg(A.vs + e));
    const double drda = drho_dalpha(__ldg(A.vp + e));
    double k = 0.0, d = 0.0;
    for (int ip = 0; ip < P; ++ip) {
      const double a = __ldg(as + ip), b = __ldg(ad + ip);
      const double s0 = __ldg(svs + ip), s1 = __ldg(svp + ip), s2 = __ldg(srho + ip);
      // ker - a*svs - a*svp*dab - a*srho*drda*dab, left to right (:229-232)
      k = __dsub_rn(k, __dmul_rn(a, s0));
      k = __dsub_rn(k, __dmul_rn(__dmul_rn(a, s1), dab));
      k = __dsub_rn(k, __dmul_rn(__dmul_rn(__dmul_rn(a, s2), drda), dab));
      d = __dsub_rn(d, __dmul_rn(b, s0));
      d = __dsub_rn(d, __dmul_rn(__dmul_rn(b, s1), dab));
      d = __dsub_rn(d, __dmul_rn(__dmul_rn(__dmul_rn(b, s2), drda), dab));
    }
    A.ker[e] = k;
    A.kd[e] = d;
  }
}

void launch_combine(int P, int nx, int ny, int nz, const double* adj_s,
                    const double* adj_density, const double* sen_vs, const double* sen_vp,
                    const double* sen_rho, const double* vs3d, const double* vp3d,
                    int use_alpha_beta_rho, int rho_scaling, double* ker, double* ker_density,
                    cudaStream_t st) {
  const size_t N3 = (size_t)nx * ny * nz;
  if (!N3) return;
  CombineArgs A{P,      nx,     ny,      nz,   rho_scaling, adj_s, adj_density, sen_vs,
                sen_vp, sen_rho, vs3d,   vp3d, ker,         ker_density};
  const unsigned grid = (unsigned)((N3 + 127) / 128);
  if (use_alpha_beta_rho) k_combine<true><<<grid, 128, 0, st>>>(A);
  else k_combine<false><<<grid, 128, 0, st>>>(A);
}

// ---------------------------------------------------------------------------
// Post-processing.
// ---------------------------------------------------------------------------
struct PrepArgs {
  int nker;
  long long N3;
  double *ker, *scaled;
  const double* kd;
  const unsigned long long* absmax;
  double coe, dx, dy, dz;
};

// max |ker_density(iker, :, :, :)| (non-negative doubles order as integers).
__global__ void k_absmax(int nker, long long N3, const double* kd, unsigned long long* out) {
  const int iker = blockIdx.y;
  unsigned long long m = 0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < N3;
       e += (long long)gridDim.x * blockDim.x) {
    const unsigned long long v =
        (unsigned long long)__double_as_longlong(fabs(kd[iker + (long long)nker * e]));
    m = v > m ? v : m;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, m, o);
    m = x > m ? x : m;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out + iker, m);
}

// regularize_ker_density (src/acqui.f90:288-303) applied as :270-273, then
// the scaled kernel of inv_grid_iso's terms: adj*dx*dy*dz (:1603).
template <bool PRECOND>
__global__ void __launch_bounds__(128) k_post_prep(PrepArgs A) {
  const int iker = blockIdx.y;
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= A.N3) return;
  const long long q = iker + (long long)A.nker * e;
  double v = A.ker[q];
  if (PRECOND) {
    const double mx = __longlong_as_double((long long)A.absmax[iker]);
    double p = __ddiv_rn(fabs(A.kd[q]), mx);
    p = p < 1.0e-4 ? 0.0 : __ddiv_rn(1.0, pow(p, A.coe));  // precond_thres, shared_par.f90:23
    v = __dmul_rn(v, p);
    A.ker[q] = v;
  }
  A.scaled[iker * A.N3 + e] = __dmul_rn(__dmul_rn(__dmul_rn(v, A.dx), A.dy), A.dz);
}

// Which resolution (0 walking up, 1 walking down) the reference's walk gives
// a node on an inversion-grid plane.  inv_grid_iso loops j = 2..ny-1,
// i = 2..nx-1, k = 2..nz-1 (0-based first = 1), inv2fwd_iso j = 1..ny,
// i = 1..nx, k = 1..nz (first = 0); each set restarts the walk at cell 1.
// x: the first node of every row after the first is reached from the
// previous row's last x (from above), unless the row has one node.  z: the
// same for the first node of every column after the set's first column.
// y only increases.
__device__ __forceinline__ int rule_x(int i, int j, int first, int nrow) {
  return (j != first && i == first && nrow >= 2) ? 1 : 0;
}
__device__ __forceinline__ int rule_z(int k, int i, int j, int first, int ncol) {
  return (!(i == first && j == first) && k == first && ncol >= 2) ? 1 : 0;
}

// inv_grid_iso (src/eikon_solver_2d.f90:1541-1614), first pass: one thread
// per (set, interior model node) evaluates the node's cell (the walk's
// resolution, rule_x / rule_z) and its eight terms scaled * wt(n), each
// rounded as the reference rounds adj*dx*dy*dz*wt(n) (:1603, the trilinear
// weights of :1527-1534), into terms[(s*Nint + q)*8 + n] with q the node's
// position in the reference's loop order (j, i, k); the cell goes to
// cells[s*Nint + q] packed as cx | cy << 10 | cz << 20.
// grid (ceil(nset*Nint/128), nker).
__global__ void __launch_bounds__(128) k_inv_terms(ProjDev P, const double* scaled,
                                                   double* terms, int* cells) {
  const int nx = P.nx, ny = P.ny, nz = P.nz;
  const int mx = nx - 2, my = ny - 2, mz = nz - 2;
  const long long Nint = (long long)mx * my * mz;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= P.nset * Nint) return;
  const int iker = blockIdx.y;
  const int s = (int)(t / Nint);
  const long long q = t - s * Nint;
  const int k = 1 + (int)(q % mz), i = 1 + (int)((q / mz) % mx), j = 1 + (int)(q / ((long long)mz * mx));
  const int ux = rule_x(i, j, 1, mx), uz = rule_z(k, i, j, 1, mz);
  const int cx = __ldg(P.cell[0] + (size_t)(2 * s + ux) * nx + i);
  const int cy = __ldg(P.cell[1] + (size_t)(2 * s) * ny + j);
  const int cz = __ldg(P.cell[2] + (size_t)(2 * s + uz) * nz + k);
  const double wx = __ldg(P.w[0] + (size_t)(2 * s + ux) * nx + i);
  const double wy = __ldg(P.w[1] + (size_t)(2 * s) * ny + j);
  const double wz = __ldg(P.w[2] + (size_t)(2 * s + uz) * nz + k);
  const double ox = __dsub_rn(1.0, wx), oy = __dsub_rn(1.0, wy), oz = __dsub_rn(1.0, wz);
  const double xy11 = __dmul_rn(ox, oy), xy12 = __dmul_rn(ox, wy);
  const double xy22 = __dmul_rn(wx, wy), xy21 = __dmul_rn(wx, oy);
  const double A = __ldg(scaled + (size_t)iker * nx * ny * nz + i + (size_t)nx * (j + (size_t)ny * k));
  double* o = terms + ((size_t)iker * P.nset + s) * 8 * Nint + q;  // corner-major
  o[0 * Nint] = __dmul_rn(A, __dmul_rn(xy11, oz));
  o[1 * Nint] = __dmul_rn(A, __dmul_rn(xy12, oz));
  o[2 * Nint] = __dmul_rn(A, __dmul_rn(xy22, oz));
  o[3 * Nint] = __dmul_rn(A, __dmul_rn(xy21, oz));
  o[4 * Nint] = __dmul_rn(A, __dmul_rn(xy11, wz));
  o[5 * Nint] = __dmul_rn(A, __dmul_rn(xy12, wz));
  o[6 * Nint] = __dmul_rn(A, __dmul_rn(xy22, wz));
  o[7 * Nint] = __dmul_rn(A, __dmul_rn(xy21, wz));
  if (iker == 0) cells[t] = cx | (cy << 10) | (cz << 20);
}

// Second pass: one thread per inversion node (set, a, b, c) adds, in the
// reference's loop order, the term of every interior node whose cell has
// the inversion node as a corner: one FP64 add per term, the chain the
// reference's scatter forms for gk(m).  Corner n of the node in a cell
// (cx, cy, cz) follows from da = a - cx, db = b - cy, dc = c - cz (each 0
// or 1): n = 4 dc + {0, 3, 1, 2}[da + 2 db] (:1583-1600).  Terms are
// corner-major, so the terms of one (j, i) line are two contiguous runs.
// When the node's z range has at most kGatherK model nodes, membership and
// dc along z come from bit masks built once per thread and the terms of a
// (j, i) line are loaded into registers a line ahead, so that only the adds
// form a chain.
// K: register window along z.  grid (ceil(nset*ninv/128), nker).
__device__ __forceinline__ int corner_xy(int da, int db) {
  return (0x2130 >> (4 * (da + 2 * db))) & 0xf;
}

constexpr int kGatherK = 16;  // largest z range held in registers
template <int K>
struct GatherLine {
  double v[K];
  unsigned in;
};

template <int K>
__global__ void __launch_bounds__(128) k_inv_gather(ProjDev P, const double* terms,
                                                    const int* cells, double* gk) {
  const int ninv = P.ninv[0] * P.ninv[1] * P.ninv[2];
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
  // Every lane stays to the end (the warp shuffles below use the full
  // mask); lanes past the last node work on node 0 and store nothing.
  const bool active = t0 < P.nset * ninv;
  const int t = active ? t0 : 0;
  const int iker = blockIdx.y;
  const int s = t / ninv, r = t - s * ninv;
  const int a = r % P.ninv[0], b = (r / P.ninv[0]) % P.ninv[1], c = r / (P.ninv[0] * P.ninv[1]);
  const int nx = P.nx, ny = P.ny, nz = P.nz;
  const int mx = nx - 2, mz = nz - 2;
  const long long Nint = (long long)mx * (ny - 2) * mz;
  const int2 rx = P.rng[0][s * P.ninv[0] + a];
  const int2 ry = P.rng[1][s * P.ninv[1] + b];
  const int2 rz = P.rng[2][s * P.ninv[2] + c];
  const double* tm = terms + ((size_t)iker * P.nset + s) * 8 * Nint;
  const int* cxs = P.cell[0] + (size_t)(2 * s) * nx;
  const int* cys = P.cell[1] + (size_t)(2 * s) * ny;
  const int* czs = P.cell[2] + (size_t)(2 * s) * nz;
  double sum = 0.0;
  const int nk = rz.y - rz.x + 1;
  if (__all_sync(0xffffffffu, nk <= K)) {  // warp-uniform choice
    // z membership / dc bits for the walk-up resolution, and the walk-down
    // resolution of the first interior node (k = 1) where it applies
    unsigned zin = 0, zdc = 0;
    for (int k = rz.x; k <= rz.y; ++k) {
      const int dc = c - __ldg(czs + k);
      if ((unsigned)dc <= 1u) {
        zin |= 1u << (k - rz.x);
        zdc |= (unsigned)dc << (k - rz.x);
      }
    }
    const bool k1u = rz.x == 1 && mz >= 2;
    const int dc1u = k1u ? c - __ldg(czs + nz + 1) : 0;
    const unsigned zin1 = (zin & ~1u) | ((unsigned)dc1u <= 1u ? 1u : 0u);
    const unsigned zdc1 = (zdc & ~1u) | (dc1u == 1 ? 1u : 0u);
    // Lines (j, i) in loop order, L = (j - ry.x) * nxl + (i - rx.x); every
    // lane runs the warp's longest list (no divergent branches: lines that
    // are not the lane's, or whose cell misses the node, add nothing), and
    // the loads of the next line are issued before the adds of the current.
    const int nxl = rx.y - rx.x + 1, nyl = ry.y - ry.x + 1;
    const int nlines = (nxl > 0 && nyl > 0) ? nxl * nyl : 0;
    int maxl = nlines;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) maxl = max(maxl, __shfl_xor_sync(0xffffffffu, maxl, o));
    auto load = [&](int L, GatherLine<K>& G) {
      const int Lc = L < nlines ? L : 0;
      const int jj = ry.x + (nxl > 0 ? Lc / nxl : 0), ii = rx.x + (nxl > 0 ? Lc % nxl : 0);
      const int jc = min(max(jj, 1), ny - 2), ic = min(max(ii, 1), nx - 2);
      const int db = b - __ldg(cys + jc);
      const int u = rule_x(ic, jc, 1, mx);
      const int da = a - __ldg(cxs + u * nx + ic);
      const bool ok = L < nlines && (unsigned)db <= 1u && (unsigned)da <= 1u;
      const double* lo = tm + (size_t)(ok ? corner_xy(da, db) : 0) * Nint +
                         ((long long)(jc - 1) * mx + (ic - 1)) * mz - 1 + rz.x;
      const bool down1 = k1u && !(ic == 1 && jc == 1);
      G.in = ok ? (down1 ? zin1 : zin) : 0u;
      const unsigned dcb = down1 ? zdc1 : zdc;
#pragma unroll
      for (int kk = 0; kk < K; ++kk)
        G.v[kk] = kk < nk ? __ldg(lo + kk + ((dcb >> kk) & 1u ? 4 * Nint : 0)) : 0.0;
    };
    GatherLine<K> cur, nxt;
    load(0, cur);
    for (int L = 0; L < maxl; ++L) {
      load(L + 1, nxt);
#pragma unroll
      for (int kk = 0; kk < K; ++kk)
        if ((cur.in >> kk) & 1u) sum = __dadd_rn(sum, cur.v[kk]);
      cur = nxt;
    }
  } else {
    for (int j = ry.x; j <= ry.y; ++j) {
      const int db = b - __ldg(cys + j);
      if ((unsigned)db > 1u) continue;
      for (int i = rx.x; i <= rx.y; ++i) {
        const int u = rule_x(i, j, 1, mx);
        const int da = a - __ldg(cxs + u * nx + i);
        if ((unsigned)da > 1u) continue;
        const int nxy = corner_xy(da, db);
        const long long q0 = ((long long)(j - 1) * mx + (i - 1)) * mz - 1;
        for (int k = rz.x; k <= rz.y; ++k) {
          const int v = rule_z(k, i, j, 1, mz);
          const int dc = c - __ldg(czs + v * nz + k);
          if ((unsigned)dc > 1u) continue;
          sum = __dadd_rn(sum, __ldg(tm + (size_t)(4 * dc + nxy) * Nint + q0 + k));
        }
      }
    }
  }
  (void)cells;
  if (active) gk[(size_t)iker * P.nset * ninv + t] = sum;
}

// inv2fwd_iso (src/eikon_solver_2d.f90:1617-1691): one thread per model
// node, the sets in order, the eight corner terms in the reference's order
// n = 1..8.  With SCALE, then update / nset / chi0 and gradient_s +=
// update * weight (src/acqui.f90:280-281); without, update is written.
// grid (ceil(N3/128), nker).
template <bool SCALE>
__global__ void __launch_bounds__(128) k_inv2fwd(ProjDev P, const double* gk, int nker,
                                                 double* out, double chi0, double weight) {
  const int nx = P.nx, ny = P.ny, nz = P.nz;
  const long long N3 = (long long)nx * ny * nz;
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= N3) return;
  const int iker = blockIdx.y;
  const int i = (int)(e % nx), j = (int)((e / nx) % ny), k = (int)(e / ((long long)nx * ny));
  const int nxi = P.ninv[0], nyi = P.ninv[1];
  const int ninv = nxi * nyi * P.ninv[2];
  const int ux = rule_x(i, j, 0, nx), uz = rule_z(k, i, j, 0, nz);
  double upd = 0.0;
  for (int s = 0; s < P.nset; ++s) {
    const int cxv = __ldg(P.cell[0] + (size_t)(2 * s + ux) * nx + i);
    const int cyv = __ldg(P.cell[1] + (size_t)(2 * s) * ny + j);
    const int czv = __ldg(P.cell[2] + (size_t)(2 * s + uz) * nz + k);
    const double wx = __ldg(P.w[0] + (size_t)(2 * s + ux) * nx + i);
    const double wy = __ldg(P.w[1] + (size_t)(2 * s) * ny + j);
    const double wz = __ldg(P.w[2] + (size_t)(2 * s + uz) * nz + k);
    const double ox = __dsub_rn(1.0, wx), oy = __dsub_rn(1.0, wy), oz = __dsub_rn(1.0, wz);
    const double xy11 = __dmul_rn(ox, oy), xy12 = __dmul_rn(ox, wy);
    const double xy22 = __dmul_rn(wx, wy), xy21 = __dmul_rn(wx, oy);
    const double* g = gk + ((size_t)iker * P.nset + s) * ninv;
    const int m = cxv + nxi * (cyv + nyi * czv);
    const int mz = nxi * nyi;
    double val = 0.0;
    val = __dadd_rn(val, __dmul_rn(__dmul_rn(xy11, oz), __ldg(g + m)));
    val = __dadd_rn(val, __dmul_rn(__dmul_rn(xy12, oz), __ldg(g + m + nxi)));
    val = __dadd_rn(val, __dmul_rn(__dmul_rn(xy22, oz), __ldg(g + m + nxi + 1)));
    val = __dadd_rn(val, __dmul_rn(__dmul_rn(xy21, oz), __ldg(g + m + 1)));
    val = __dadd_rn(val, __dmul_rn(__dmul_rn(xy11, wz), __ldg(g + m + mz)));
    val = __dadd_rn(val, __dmul_rn(__dmul_rn(xy12, wz), __ldg(g + m + mz + nxi)));
    val = __dadd_rn(val, __dmul_rn(__dmul_rn(xy22, wz), __ldg(g + m + mz + nxi + 1)));
    val = __dadd_rn(val, __dmul_rn(__dmul_rn(xy21, wz), __ldg(g + m + mz + 1)));
    upd = __dadd_rn(upd, val);
  }
  if (SCALE) {
    const double u = __ddiv_rn(__ddiv_rn(upd, (double)P.nset), chi0);
    const long long q = iker + (long long)nker * e;
    out[q] = __dadd_rn(out[q], __dmul_rn(u, weight));
  } else {
    out[e] = upd;
  }
}

void launch_gather(const ProjDev& P, const double* terms, const int* cells, double* gk, int nker,
                   cudaStream_t st) {
  const int ninv = P.ninv[0] * P.ninv[1] * P.ninv[2];
  const dim3 g((P.nset * ninv + 127) / 128, nker);
  k_inv_gather<kGatherK><<<g, 128, 0, st>>>(P, terms, cells, gk);
}

void launch_post_process(const ProjDev& P, int nker, double* ker, const double* ker_density,
                         double kdensity_coe, double* scaled, double* terms, int* cells,
                         double* gk, unsigned long long* absmax, double chi0, double weight,
                         double* gradient_s, cudaStream_t st) {
  const long long N3 = (long long)P.nx * P.ny * P.nz;
  const int ninv = P.ninv[0] * P.ninv[1] * P.ninv[2];
  PrepArgs A{nker, N3, ker, scaled, ker_density, absmax, kdensity_coe, P.dx, P.dy, P.dz};
  const dim3 g3((unsigned)((N3 + 127) / 128), nker);
  if (kdensity_coe > 0) {
    cudaMemsetAsync(absmax, 0, nker * sizeof(unsigned long long), st);
    k_absmax<<<dim3(152, nker), 256, 0, st>>>(nker, N3, ker_density, absmax);
    k_post_prep<true><<<g3, 128, 0, st>>>(A);
  } else {
    k_post_prep<false><<<g3, 128, 0, st>>>(A);
  }
  const long long Nint = (long long)(P.nx - 2) * (P.ny - 2) * (P.nz - 2);
  if (Nint > 0) {
    k_inv_terms<<<dim3((unsigned)((P.nset * Nint + 127) / 128), nker), 128, 0, st>>>(
        P, scaled, terms, cells);
    launch_gather(P, terms, cells, gk, nker, st);
  } else {
    cudaMemsetAsync(gk, 0, (size_t)nker * P.nset * ninv * sizeof(double), st);
  }
  k_inv2fwd<true><<<g3, 128, 0, st>>>(P, gk, nker, gradient_s, chi0, weight);
}

void launch_inv_grid(const ProjDev& P, const double* adj, double* scaled, double* terms,
                     int* cells, double* gk, cudaStream_t st) {
  const long long N3 = (long long)P.nx * P.ny * P.nz;
  PrepArgs A{1, N3, const_cast<double*>(adj), scaled, nullptr, nullptr, 0.0, P.dx, P.dy, P.dz};
  k_post_prep<false><<<(unsigned)((N3 + 127) / 128), 128, 0, st>>>(A);
  const int ninv = P.ninv[0] * P.ninv[1] * P.ninv[2];
  const long long Nint = (long long)(P.nx - 2) * (P.ny - 2) * (P.nz - 2);
  if (Nint > 0) {
    k_inv_terms<<<dim3((unsigned)((P.nset * Nint + 127) / 128), 1), 128, 0, st>>>(P, scaled,
                                                                                 terms, cells);
    launch_gather(P, terms, cells, gk, 1, st);
  } else {
    cudaMemsetAsync(gk, 0, (size_t)P.nset * ninv * sizeof(double), st);
  }
}

void launch_inv2fwd(const ProjDev& P, const double* gk, double* update, cudaStream_t st) {
  const long long N3 = (long long)P.nx * P.ny * P.nz;
  k_inv2fwd<false><<<dim3((unsigned)((N3 + 127) / 128), 1), 128, 0, st>>>(P, gk, 1, update, 1.0,
                                                                          1.0);
}

}  // namespace sgb
