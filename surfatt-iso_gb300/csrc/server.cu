// server.cu -- the serving loop: gradient evaluations, line-search trials and
// forward-only runs submitted as requests, admitted by an HBM budget and run
// concurrently on one GPU.
//
// Device memory: one allocation of the budget at creation, sub-allocated
// first-fit (256-byte aligned, coalescing).  Models (grids, surface metric,
// velocity and their per-period precompute) and work lists (sources,
// receivers, observed times: the station tables) stay resident across
// requests.  A request names a work list, optionally carries its own velocity
// model (a line-search trial or the next inversion iterate), and gets its own
// stream, outputs and solve workspace from the arena.
//
// Continuous batching: a scheduler thread admits queued requests in arrival
// order whenever an in-flight slot and enough arena memory are free, and
// launches each on its own stream; the solve kernels of admitted requests
// share the SMs as their blocks retire.  Completion is detected with event
// queries; results are copied to host memory and the request's memory is
// returned to the arena at once.  Each request's result is independent of
// what runs beside it (deterministic per-solve work and ordered sums).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

#include "../../include/surfatt_gb300.h"
#include "launch.cuh"

using namespace sgb;

namespace {

constexpr size_t kAlign = 256;
inline size_t up256(size_t b) { return (b + kAlign - 1) / kAlign * kAlign; }

// First-fit sub-allocator over one device allocation.
class Arena {
 public:
  int init(size_t bytes) {
    size_ = up256(bytes);
    if (cudaMalloc(&base_, size_) != cudaSuccess) {
      cudaGetLastError();
      base_ = nullptr;
      return ST_OOM;
    }
    free_[0] = size_;
    return ST_OK;
  }
  ~Arena() {
    if (base_) cudaFree(base_);
  }
  bool alloc(size_t bytes, size_t* off) {
    bytes = up256(std::max<size_t>(bytes, 1));
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        const size_t o = it->first, rem = it->second - bytes;
        free_.erase(it);
        if (rem) free_[o + bytes] = rem;
        *off = o;
        used_ += bytes;
        peak_ = std::max(peak_, used_);
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = up256(std::max<size_t>(bytes, 1));
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  char* ptr(size_t off) const { return static_cast<char*>(base_) + off; }
  size_t size() const { return size_; }
  size_t used() const { return used_; }
  size_t peak() const { return peak_; }

 private:
  void* base_ = nullptr;
  size_t size_ = 0, used_ = 0, peak_ = 0;
  std::map<size_t, size_t> free_;
};

// Lays out typed sub-buffers in one chunk: first pass sizes, second carves.
struct Carver {
  size_t off = 0;
  char* base = nullptr;
  template <class T>
  T* take(size_t n) {
    off = up256(off);
    T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
    off += std::max<size_t>(n, 1) * sizeof(T);
    return p;
  }
};

struct PeriodArrays {
  double *xdeg, *ydeg, *xs, *ys, *cosy, *siny, *A, *B, *C, *V, *a, *b, *c, *fun, *f2, *disx, *disy;
  float* f32;
  double* isv;
  float4 *p4a, *p4b;
  PeriodDev* periods;
  long long *goff;
  int *nx, *ny;
};

void carve_periods(Carver& cv, long long nxs, long long nys, long long NC, int np,
                   PeriodArrays* a) {
  a->xdeg = cv.take<double>(nxs);
  a->ydeg = cv.take<double>(nys);
  a->xs = cv.take<double>(nxs);
  a->ys = cv.take<double>(nys);
  a->cosy = cv.take<double>(nys);
  a->siny = cv.take<double>(nys);
  a->A = cv.take<double>(NC);
  a->B = cv.take<double>(NC);
  a->C = cv.take<double>(NC);
  a->V = cv.take<double>(NC);
  a->a = cv.take<double>(NC);
  a->b = cv.take<double>(NC);
  a->c = cv.take<double>(NC);
  a->fun = cv.take<double>(NC);
  a->f2 = cv.take<double>(NC);
  a->disx = cv.take<double>(NC);
  a->disy = cv.take<double>(NC);
  a->f32 = cv.take<float>(6 * NC);
  a->isv = cv.take<double>(2 * NC);
  a->p4a = cv.take<float4>(2 * NC);  // 32-byte records
  a->p4b = a->p4a ? a->p4a + 1 : nullptr;
  a->periods = cv.take<PeriodDev>(np);
  a->goff = cv.take<long long>(np);
  a->nx = cv.take<int>(np);
  a->ny = cv.take<int>(np);
}

struct Model {
  int id = 0;
  size_t off = 0, bytes = 0;
  int nperiod = 0;
  long long ncell = 0, nxs = 0, nys = 0;
  std::vector<int> nx, ny;
  std::vector<long long> goff, xoff, yoff;
  std::vector<double> dx, dy;
  PeriodArrays d{};
  int refs = 0;
};

struct WorkList {
  int id = 0, model = 0;
  size_t off = 0, bytes = 0;
  int nsolve = 0, npath = 0, nrec_total = 0;
  long long kslot_total = 0;
  int *pidx, *rec_off, *nrec, *path, *order, *plist_off, *plist;
  double *srcx, *srcy, *recx, *recy, *tt, *weight;
  long long* kslot;
  std::vector<int> pidx_h;  // host copy: team classes of the launch plan
};

enum ReqState { RQ_PENDING = 0, RQ_RUNNING = 1, RQ_DONE = 2 };

struct Request {
  long long ticket = 0;
  int wl = 0, mode = 2, prec = 0;
  std::vector<double> svel;  // velocity override (empty: the model's)
  int state = RQ_PENDING;
  int status = ST_OK;
  std::chrono::steady_clock::time_point t_submit, t_start, t_done;
  size_t off = 0, bytes = 0;
  cudaStream_t st = nullptr;
  ClassStreams cs;  // side streams of the row kernel's team classes
  cudaEvent_t done = nullptr;
  // device buffers (in the request's chunk)
  PeriodArrays d{};
  double *tekio, *wgt, *ttfwd, *chis, *chi, *kc, *kcd, *adj, *adjd, *fupd, *aupd, *ws;
  int *status_d, *fit, *ait, *queue;
  LaunchPlan plan;
  EvalShape shape;
  // host results
  std::vector<double> h_adj, h_adjd, h_tt;
  std::vector<int> h_status, h_fit, h_ait;
  double h_chi = 0;
};

}  // namespace

struct surfatt_server {
  int device = 0;
  int max_inflight = 4;
  Arena arena;
  std::mutex mu;
  std::condition_variable cv_done, cv_work;
  std::map<int, std::unique_ptr<Model>> models;
  std::map<int, std::unique_ptr<WorkList>> lists;
  std::map<long long, std::unique_ptr<Request>> reqs;
  std::deque<long long> pending;
  std::vector<long long> inflight;
  int next_model = 1, next_list = 1;
  long long next_ticket = 1;
  bool stop = false;
  std::thread worker;
  // statistics
  std::vector<double> lat_ms;
  long long submitted = 0, completed = 0, failed = 0, solves = 0;
  int inflight_peak = 0;
  std::chrono::steady_clock::time_point t_first, t_last;
  bool any = false;
};

namespace {

// Per-period precompute of a model (or of a request's velocity override)
// from the model's metric and the given velocity.
int prep_periods(const Model& m, const PeriodArrays& src_axes, const PeriodArrays& out,
                 const double* V, cudaStream_t st) {
  std::vector<PrepIn> ins(m.nperiod);
  std::vector<PrepOut> outs(m.nperiod);
  for (int p = 0; p < m.nperiod; ++p) {
    const long long g = m.goff[p];
    ins[p] = PrepIn{m.nx[p], m.ny[p], 1, src_axes.xdeg + m.xoff[p], src_axes.ydeg + m.yoff[p],
              src_axes.A + g, src_axes.B + g, src_axes.C + g, V + g, 1};
    auto ax = [](double* b, long long o) { return b ? b + o : nullptr; };
    outs[p] = PrepOut{ax(out.xs, m.xoff[p]), ax(out.ys, m.yoff[p]), ax(out.cosy, m.yoff[p]),
                      ax(out.siny, m.yoff[p]),
                      out.a + g, out.b + g, out.c + g, out.fun + g, out.f2 + g, out.disx + g,
                      out.disy + g, out.f32 + 6 * g, out.isv + 2 * g, out.p4a + 2 * g,
                      out.p4b + 2 * g};
  }
  launch_prep_batch(ins.data(), outs.data(), m.nperiod, st);
  return cudaGetLastError() == cudaSuccess ? ST_OK : ST_CUDA_ERROR;
}

std::vector<PeriodDev> period_descs(const Model& m, const PeriodArrays& axes,
                                    const PeriodArrays& f) {
  std::vector<PeriodDev> out(m.nperiod);
  for (int p = 0; p < m.nperiod; ++p) {
    PeriodDev& P = out[p];
    const long long g = m.goff[p];
    P.nx = m.nx[p];
    P.ny = m.ny[p];
    P.lonlat = 1;
    P.dx = m.dx[p];
    P.dy = m.dy[p];
    P.xs = axes.xs + m.xoff[p];
    P.ys = axes.ys + m.yoff[p];
    P.xdeg = axes.xdeg + m.xoff[p];
    P.ydeg = axes.ydeg + m.yoff[p];
    P.cosy = axes.cosy + m.yoff[p];
    P.siny = axes.siny + m.yoff[p];
    P.a = f.a + g;
    P.b = f.b + g;
    P.c = f.c + g;
    P.fun = f.fun + g;
    P.f2 = f.f2 + g;
    P.disx = f.disx + g;
    P.disy = f.disy + g;
    P.svel = f.V + g;
    P.goff = g;
    P.f32 = f.f32 + 6 * g;
    P.isv = f.isv + 2 * g;
    P.p4a = f.p4a + 2 * g;
    P.p4b = f.p4b + 2 * g;
  }
  return out;
}

// Admit one request: carve its chunk, upload / precompute, enqueue.
int start_request(surfatt_server* S, Request& r) {
  WorkList& L = *S->lists[r.wl];
  Model& M = *S->models[L.model];
  const bool own_vel = !r.svel.empty();
  r.shape.from_grids(M.nx.data(), M.ny.data(), M.goff.data(), M.nperiod, L.nsolve, L.npath,
                     L.pidx_h.data());
  // The row kernel's variant 4: work items, and grids of more than 128 rows
  // swept in strips by one warp.  On the serving workload (40 requests, 64^2
  // to 512^2) it serves 15,800 solves/s at p99 141 ms, against 14,100 at
  // 195 ms with teams on whole solves and 13,600 at 207 ms with teams on
  // items: the tall grids' requests hold a third of the warps and their
  // adjoint fields run side by side.
  KernelChoice choice;
  choice.variant = 4;
  int e = plan_evaluation(r.shape, r.prec, S->device, 0, &r.plan, choice);
  if (e) return e;
  auto layout = [&](Carver& cv) {
    if (own_vel) carve_periods(cv, M.nxs, M.nys, M.ncell, M.nperiod, &r.d);
    const int nr = std::max(1, L.nrec_total), ns = std::max(1, L.nsolve);
    r.tekio = cv.take<double>(nr);
    r.wgt = cv.take<double>(nr);
    r.ttfwd = cv.take<double>(std::max(1, L.npath));
    r.chis = cv.take<double>(ns);
    r.chi = cv.take<double>(1);
    r.kc = cv.take<double>(L.kslot_total);
    r.kcd = cv.take<double>(r.mode == 3 ? L.kslot_total : 1);
    r.adj = cv.take<double>(M.ncell);
    r.adjd = cv.take<double>(M.ncell);
    r.fupd = cv.take<double>(ns);
    r.aupd = cv.take<double>(ns);
    r.status_d = cv.take<int>(ns);
    r.fit = cv.take<int>(ns);
    r.ait = cv.take<int>(ns);
    r.queue = cv.take<int>(kTeamClasses);
    r.ws = cv.take<double>((size_t)plan_ws_doubles(r.plan, L.nsolve));
  };
  Carver sizer;
  layout(sizer);
  size_t off = 0;
  if (!S->arena.alloc(sizer.off, &off)) return ST_OOM;  // nothing held: may retry later
  r.off = off;
  r.bytes = sizer.off;
  Carver cv;
  cv.base = S->arena.ptr(r.off);
  layout(cv);
  if (cudaStreamCreateWithFlags(&r.st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&r.done, cudaEventDisableTiming) != cudaSuccess)
    return ST_CUDA_ERROR;
  if (r.plan.classes > 1 && r.cs.create() != ST_OK) return ST_CUDA_ERROR;
  const PeriodDev* periods = M.d.periods;
  if (own_vel) {
    // the request's velocity with the model's axes and metric
    if (cudaMemcpyAsync(r.d.V, r.svel.data(), M.ncell * sizeof(double), cudaMemcpyHostToDevice,
                        r.st) != cudaSuccess)
      return ST_CUDA_ERROR;
    // the model's axes stay as they are (other requests read them)
    PeriodArrays outs = r.d;
    outs.xs = outs.ys = outs.cosy = outs.siny = nullptr;
    e = prep_periods(M, M.d, outs, r.d.V, r.st);
    if (e) return e;
    std::vector<PeriodDev> pd = period_descs(M, M.d, outs);
    if (cudaMemcpyAsync(r.d.periods, pd.data(), pd.size() * sizeof(PeriodDev),
                        cudaMemcpyHostToDevice, r.st) != cudaSuccess)
      return ST_CUDA_ERROR;
    periods = r.d.periods;
  }
  EvalDev dev;
  BatchArgs& A = dev.args;
  A.periods = periods;
  A.nsolve = L.nsolve;
  A.order = L.order;
  A.pidx = L.pidx;
  A.srcx = L.srcx;
  A.srcy = L.srcy;
  A.rec_off = L.rec_off;
  A.nrec = L.nrec;
  A.recx = L.recx;
  A.recy = L.recy;
  A.tt = L.tt;
  A.weight = L.weight;
  A.path = L.path;
  A.kslot = L.kslot;
  A.tekio = r.tekio;
  A.wgt_eff = r.wgt;
  A.tt_fwd = r.ttfwd;
  A.chi = r.chis;
  A.kcontrib = r.kc;
  A.kcontrib_den = r.kcd;
  A.status = r.status_d;
  A.fwd_iters = r.fit;
  A.adj_iters = r.ait;
  A.fwd_updates = r.fupd;
  A.adj_updates = r.aupd;
  A.Tout = nullptr;
  dev.plist_off = L.plist_off;
  dev.plist = L.plist;
  dev.goff = M.d.goff;
  dev.nx = M.d.nx;
  dev.ny = M.d.ny;
  dev.chi_total = r.chi;
  dev.adj_s = r.adj;
  dev.adj_density = r.adjd;
  const int n = enqueue_evaluation(r.shape, dev, r.plan, r.mode, r.prec, r.ws, r.queue, r.st,
                                   nullptr, nullptr, &r.cs);
  if (n < 0) return -n;
  if (cudaEventRecord(r.done, r.st) != cudaSuccess) return ST_CUDA_ERROR;
  return ST_OK;
}

void finish_request(surfatt_server* S, Request& r) {
  WorkList& L = *S->lists[r.wl];
  Model& M = *S->models[L.model];
  r.h_adj.assign(M.ncell, 0.0);
  r.h_adjd.assign(M.ncell, 0.0);
  r.h_tt.assign(L.npath, 0.0);
  r.h_status.assign(L.nsolve, 0);
  r.h_fit.assign(L.nsolve, 0);
  r.h_ait.assign(L.nsolve, 0);
  bool ok = true;
  auto cp = [&](void* dst, const void* src, size_t bytes) {
    if (bytes && cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, r.st) != cudaSuccess)
      ok = false;
  };
  if (r.status == ST_OK) {
    if (r.mode >= 2) cp(r.h_adj.data(), r.adj, M.ncell * sizeof(double));
    if (r.mode == 3) cp(r.h_adjd.data(), r.adjd, M.ncell * sizeof(double));
    cp(r.h_tt.data(), r.ttfwd, L.npath * sizeof(double));
    cp(&r.h_chi, r.chi, sizeof(double));
    cp(r.h_status.data(), r.status_d, L.nsolve * sizeof(int));
    cp(r.h_fit.data(), r.fit, L.nsolve * sizeof(int));
    cp(r.h_ait.data(), r.ait, L.nsolve * sizeof(int));
    if (cudaStreamSynchronize(r.st) != cudaSuccess) ok = false;
    if (!ok) r.status = ST_CUDA_ERROR;
    for (int s = 0; s < L.nsolve && r.status == ST_OK; ++s)
      if (r.h_status[s] != ST_OK) r.status = r.h_status[s];
  } else if (r.st) {
    // a request that failed part-way may still have work queued: none of
    // it may write into the chunk once the arena hands it out again
    cudaStreamSynchronize(r.st);
    for (cudaStream_t s : r.cs.side)
      if (s) cudaStreamSynchronize(s);
    cudaGetLastError();
  }
  if (r.st) cudaStreamDestroy(r.st);
  if (r.done) cudaEventDestroy(r.done);
  r.cs.destroy();
  r.st = nullptr;
  r.done = nullptr;
  if (r.bytes) S->arena.release(r.off, r.bytes);
  r.bytes = 0;
  r.state = RQ_DONE;
  r.t_done = std::chrono::steady_clock::now();
  std::vector<double>().swap(r.svel);
  M.refs--;
  const double ms = std::chrono::duration<double, std::milli>(r.t_done - r.t_submit).count();
  S->lat_ms.push_back(ms);
  S->completed++;
  if (r.status != ST_OK && r.status != ST_NOT_CONVERGED) S->failed++;
  S->solves += L.nsolve;
  S->t_last = r.t_done;
}

void worker_loop(surfatt_server* S) {
  cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lk(S->mu);
  while (!S->stop) {
    bool progress = false;
    // completions
    for (size_t i = 0; i < S->inflight.size();) {
      Request& r = *S->reqs[S->inflight[i]];
      const cudaError_t q = cudaEventQuery(r.done);
      if (q == cudaErrorNotReady) {
        ++i;
        continue;
      }
      if (q != cudaSuccess) r.status = ST_CUDA_ERROR;
      finish_request(S, r);
      S->inflight.erase(S->inflight.begin() + i);
      progress = true;
      S->cv_done.notify_all();
    }
    // admissions, in arrival order
    while (!S->pending.empty() && (int)S->inflight.size() < S->max_inflight) {
      Request& r = *S->reqs[S->pending.front()];
      r.t_start = std::chrono::steady_clock::now();
      const int e = start_request(S, r);
      // arena full: wait for running requests to return memory (a request
      // that does not fit an idle arena can never run and fails)
      if (e == ST_OOM && r.bytes == 0 && !S->inflight.empty()) break;
      S->pending.pop_front();
      if (e != ST_OK) {
        r.status = e;
        finish_request(S, r);
        S->cv_done.notify_all();
      } else {
        r.state = RQ_RUNNING;
        S->inflight.push_back(r.ticket);
        S->inflight_peak = std::max<int>(S->inflight_peak, (int)S->inflight.size());
      }
      progress = true;
    }
    if (!progress) S->cv_work.wait_for(lk, std::chrono::microseconds(200));
  }
}

template <class T>
int upload(cudaStream_t st, T* dst, const T* src, size_t n) {
  if (!n || !src) return ST_OK;
  return cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyHostToDevice, st) == cudaSuccess
             ? ST_OK
             : ST_CUDA_ERROR;
}

double percentile(std::vector<double> v, double q) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double pos = q * (v.size() - 1);
  const size_t lo = (size_t)pos, hi = std::min(lo + 1, v.size() - 1);
  return v[lo] + (v[hi] - v[lo]) * (pos - lo);
}

}  // namespace

extern "C" {

surfatt_status_t surfatt_server_create(surfatt_server_t** out, int device, size_t budget,
                                       int max_inflight) {
  if (!out || budget == 0 || max_inflight < 1) return SURFATT_BAD_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    return SURFATT_CUDA_ERROR;
  }
  if (cudaSetDevice(device) != cudaSuccess) return SURFATT_CUDA_ERROR;
  auto* S = new surfatt_server();
  S->device = device;
  S->max_inflight = max_inflight;
  if (S->arena.init(budget) != ST_OK) {
    delete S;
    return SURFATT_OOM;
  }
  S->worker = std::thread(worker_loop, S);
  *out = S;
  return SURFATT_OK;
}

void surfatt_server_destroy(surfatt_server_t* S) {
  if (!S) return;
  {
    std::unique_lock<std::mutex> lk(S->mu);
    // drain: wait for running requests, drop pending ones
    while (!S->inflight.empty()) S->cv_done.wait_for(lk, std::chrono::milliseconds(5));
    S->stop = true;
  }
  S->cv_work.notify_all();
  S->worker.join();
  cudaSetDevice(S->device);
  delete S;
}

surfatt_status_t surfatt_server_add_model(surfatt_server_t* S, const surfatt_problem_t* pb,
                                          int* model_id) {
  if (!S || !pb || !model_id || pb->nperiod < 1) return SURFATT_BAD_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  cudaSetDevice(S->device);
  auto m = std::make_unique<Model>();
  m->nperiod = pb->nperiod;
  m->nx.assign(pb->nx, pb->nx + pb->nperiod);
  m->ny.assign(pb->ny, pb->ny + pb->nperiod);
  m->goff.assign(pb->goff, pb->goff + pb->nperiod);
  m->xoff.assign(pb->xoff, pb->xoff + pb->nperiod);
  m->yoff.assign(pb->yoff, pb->yoff + pb->nperiod);
  for (int p = 0; p < m->nperiod; ++p) {
    if (m->nx[p] < 3 || m->ny[p] < 3) return SURFATT_BAD_ARG;
    m->ncell = std::max(m->ncell, m->goff[p] + (long long)m->nx[p] * m->ny[p]);
    m->nxs = std::max(m->nxs, m->xoff[p] + m->nx[p]);
    m->nys = std::max(m->nys, m->yoff[p] + m->ny[p]);
    const double* xg = pb->xgrid + m->xoff[p];
    const double* yg = pb->ygrid + m->yoff[p];
    m->dx.push_back(xg[1] / 180.0 * PI_S - xg[0] / 180.0 * PI_S);
    m->dy.push_back(yg[1] / 180.0 * PI_S - yg[0] / 180.0 * PI_S);
  }
  Carver sizer;
  carve_periods(sizer, m->nxs, m->nys, m->ncell, m->nperiod, &m->d);
  m->bytes = sizer.off;
  if (!S->arena.alloc(m->bytes, &m->off)) return SURFATT_OOM;
  Carver cv;
  cv.base = S->arena.ptr(m->off);
  carve_periods(cv, m->nxs, m->nys, m->ncell, m->nperiod, &m->d);
  cudaStream_t st = nullptr;
  int e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess ? ST_OK : ST_CUDA_ERROR;
  const size_t NC = m->ncell;
  if (!e) e = upload(st, m->d.xdeg, pb->xgrid, m->nxs) | upload(st, m->d.ydeg, pb->ygrid, m->nys) |
              upload(st, m->d.A, pb->m11, NC) | upload(st, m->d.B, pb->m22, NC) |
              upload(st, m->d.C, pb->m12, NC) | upload(st, m->d.V, pb->svel, NC) |
              upload(st, m->d.goff, m->goff.data(), m->nperiod) |
              upload(st, m->d.nx, m->nx.data(), m->nperiod) |
              upload(st, m->d.ny, m->ny.data(), m->nperiod);
  if (!e) e = prep_periods(*m, m->d, m->d, m->d.V, st);
  std::vector<PeriodDev> pd = period_descs(*m, m->d, m->d);
  if (!e) e = upload(st, m->d.periods, pd.data(), pd.size());
  if (st) {
    if (cudaStreamSynchronize(st) != cudaSuccess) e = ST_CUDA_ERROR;
    cudaStreamDestroy(st);
  }
  if (e) {
    S->arena.release(m->off, m->bytes);
    return (surfatt_status_t)e;
  }
  m->id = S->next_model++;
  *model_id = m->id;
  S->models[m->id] = std::move(m);
  return SURFATT_OK;
}

surfatt_status_t surfatt_server_add_worklist(surfatt_server_t* S, int model_id,
                                             const surfatt_problem_t* pb, int* worklist_id) {
  if (!S || !pb || !worklist_id || pb->nsolve < 0) return SURFATT_BAD_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  auto mit = S->models.find(model_id);
  if (mit == S->models.end()) return SURFATT_BAD_ARG;
  const Model& M = *mit->second;
  cudaSetDevice(S->device);
  auto L = std::make_unique<WorkList>();
  L->model = model_id;
  L->nsolve = pb->nsolve;
  L->npath = pb->npath;
  const int ns = pb->nsolve;
  int nrt = 0;
  for (int s = 0; s < ns; ++s) {
    if (pb->pidx[s] < 0 || pb->pidx[s] >= M.nperiod || pb->nrec[s] < 0) return SURFATT_BAD_ARG;
    nrt = std::max(nrt, pb->rec_off[s] + pb->nrec[s]);
  }
  for (int r = 0; r < nrt; ++r)
    if (pb->path[r] < 0 || pb->path[r] >= pb->npath) return SURFATT_BAD_ARG;
  L->nrec_total = nrt;
  std::vector<int> order(ns), plist_off(M.nperiod + 1, 0), plist(ns);
  std::vector<long long> kslot(ns);
  std::iota(order.begin(), order.end(), 0);
  auto cells = [&](int s) { return (long long)M.nx[pb->pidx[s]] * M.ny[pb->pidx[s]]; };
  // team classes of the FP32 row kernel contiguous (largest team first),
  // then largest grids first
  auto cls = [&](int s) { return team_class_key(M.ny[pb->pidx[s]]); };
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return cls(a) != cls(b) ? cls(a) > cls(b) : cells(a) > cells(b);
  });
  L->pidx_h.assign(pb->pidx, pb->pidx + ns);
  for (int s = 0; s < ns; ++s) plist_off[pb->pidx[s] + 1]++;
  for (int p = 0; p < M.nperiod; ++p) plist_off[p + 1] += plist_off[p];
  {
    std::vector<int> fill(plist_off.begin(), plist_off.end() - 1);
    for (int s = 0; s < ns; ++s) plist[fill[pb->pidx[s]]++] = s;
  }
  long long acc = 0;
  for (int s = 0; s < ns; ++s) {
    kslot[s] = acc;
    acc += cells(s);
  }
  L->kslot_total = acc;
  auto layout = [&](Carver& cv) {
    L->pidx = cv.take<int>(ns);
    L->rec_off = cv.take<int>(ns);
    L->nrec = cv.take<int>(ns);
    L->path = cv.take<int>(nrt);
    L->order = cv.take<int>(ns);
    L->plist_off = cv.take<int>(M.nperiod + 1);
    L->plist = cv.take<int>(ns);
    L->srcx = cv.take<double>(ns);
    L->srcy = cv.take<double>(ns);
    L->recx = cv.take<double>(nrt);
    L->recy = cv.take<double>(nrt);
    L->tt = cv.take<double>(nrt);
    L->weight = cv.take<double>(nrt);
    L->kslot = cv.take<long long>(ns);
  };
  Carver sizer;
  layout(sizer);
  L->bytes = sizer.off;
  if (!S->arena.alloc(L->bytes, &L->off)) return SURFATT_OOM;
  Carver cv;
  cv.base = S->arena.ptr(L->off);
  layout(cv);
  cudaStream_t st = nullptr;
  int e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess ? ST_OK : ST_CUDA_ERROR;
  if (!e) e = upload(st, L->pidx, pb->pidx, ns) | upload(st, L->rec_off, pb->rec_off, ns) |
              upload(st, L->nrec, pb->nrec, ns) | upload(st, L->path, pb->path, nrt) |
              upload(st, L->order, order.data(), ns) |
              upload(st, L->plist_off, plist_off.data(), M.nperiod + 1) |
              upload(st, L->plist, plist.data(), ns) | upload(st, L->srcx, pb->srcx, ns) |
              upload(st, L->srcy, pb->srcy, ns) | upload(st, L->recx, pb->recx, nrt) |
              upload(st, L->recy, pb->recy, nrt) | upload(st, L->tt, pb->tt, nrt) |
              upload(st, L->weight, pb->weight, nrt) | upload(st, L->kslot, kslot.data(), ns);
  if (st) {
    if (cudaStreamSynchronize(st) != cudaSuccess) e = ST_CUDA_ERROR;
    cudaStreamDestroy(st);
  }
  if (e) {
    S->arena.release(L->off, L->bytes);
    return (surfatt_status_t)e;
  }
  L->id = S->next_list++;
  *worklist_id = L->id;
  S->lists[L->id] = std::move(L);
  return SURFATT_OK;
}

surfatt_status_t surfatt_server_submit(surfatt_server_t* S, int worklist_id, const double* svel,
                                       surfatt_mode_t mode, surfatt_precision_t prec,
                                       long long* ticket) {
  if (!S || !ticket) return SURFATT_BAD_ARG;
  if (mode != SURFATT_MODE_FORWARD && mode != SURFATT_MODE_2D && mode != SURFATT_MODE_3D)
    return SURFATT_BAD_ARG;
  if (prec != SURFATT_PREC_FP64 && prec != SURFATT_PREC_FP32) return SURFATT_BAD_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  auto lit = S->lists.find(worklist_id);
  if (lit == S->lists.end()) return SURFATT_BAD_ARG;
  Model& M = *S->models[lit->second->model];
  auto r = std::make_unique<Request>();
  r->ticket = S->next_ticket++;
  r->wl = worklist_id;
  r->mode = mode;
  r->prec = prec;
  if (svel) r->svel.assign(svel, svel + M.ncell);
  r->t_submit = std::chrono::steady_clock::now();
  if (!S->any) {
    S->t_first = r->t_submit;
    S->any = true;
  }
  M.refs++;
  *ticket = r->ticket;
  S->pending.push_back(r->ticket);
  S->reqs[r->ticket] = std::move(r);
  S->submitted++;
  lk.unlock();
  S->cv_work.notify_all();
  return SURFATT_OK;
}

surfatt_status_t surfatt_server_wait(surfatt_server_t* S, long long ticket, double timeout_s,
                                     surfatt_result_t* out, double* latency_ms) {
  if (!S) return SURFATT_BAD_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) return SURFATT_BAD_ARG;
  Request& r = *it->second;
  const auto deadline = std::chrono::steady_clock::now() +
                        std::chrono::duration_cast<std::chrono::steady_clock::duration>(
                            std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 1e9));
  while (r.state != RQ_DONE) {
    if (S->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && r.state != RQ_DONE)
      return SURFATT_TIMEOUT;
  }
  if (out) {
    if (out->adj_s) std::memcpy(out->adj_s, r.h_adj.data(), r.h_adj.size() * sizeof(double));
    if (out->adj_density)
      std::memcpy(out->adj_density, r.h_adjd.data(), r.h_adjd.size() * sizeof(double));
    if (out->chi) *out->chi = r.h_chi;
    if (out->tt_fwd) std::memcpy(out->tt_fwd, r.h_tt.data(), r.h_tt.size() * sizeof(double));
    if (out->status) std::memcpy(out->status, r.h_status.data(), r.h_status.size() * sizeof(int));
    if (out->fwd_iters) std::memcpy(out->fwd_iters, r.h_fit.data(), r.h_fit.size() * sizeof(int));
    if (out->adj_iters) std::memcpy(out->adj_iters, r.h_ait.data(), r.h_ait.size() * sizeof(int));
  }
  if (latency_ms)
    *latency_ms = std::chrono::duration<double, std::milli>(r.t_done - r.t_submit).count();
  const int st = r.status;
  S->reqs.erase(it);
  return (surfatt_status_t)st;
}

surfatt_status_t surfatt_server_stats(surfatt_server_t* S, surfatt_server_stats_t* out) {
  if (!S || !out) return SURFATT_BAD_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  out->submitted = S->submitted;
  out->completed = S->completed;
  out->failed = S->failed;
  out->solves = S->solves;
  out->p50_ms = percentile(S->lat_ms, 0.50);
  out->p99_ms = percentile(S->lat_ms, 0.99);
  out->mean_ms = S->lat_ms.empty()
                     ? 0.0
                     : std::accumulate(S->lat_ms.begin(), S->lat_ms.end(), 0.0) / S->lat_ms.size();
  const double span =
      S->any && S->completed ? std::chrono::duration<double>(S->t_last - S->t_first).count() : 0.0;
  out->span_s = span;
  out->solves_per_s = span > 0 ? (double)S->solves / span : 0.0;
  out->hbm_budget_bytes = S->arena.size();
  out->hbm_peak_bytes = S->arena.peak();
  out->inflight_peak = S->inflight_peak;
  return SURFATT_OK;
}

surfatt_status_t surfatt_server_reset_stats(surfatt_server_t* S) {
  if (!S) return SURFATT_BAD_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  S->lat_ms.clear();
  S->submitted = S->completed = S->failed = S->solves = 0;
  S->inflight_peak = 0;
  S->any = false;
  return SURFATT_OK;
}

}  // extern "C"
