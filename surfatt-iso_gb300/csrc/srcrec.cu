// srcrec.cu -- ids of a src_rec table (host) and its work list (GPU).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <unordered_map>

#include "common.cuh"
#include "srcrec.cuh"

namespace sgb {

namespace {

std::string rstrip(const std::string& s) {
  size_t n = s.size();
  while (n && s[n - 1] == ' ') --n;
  return s.substr(0, n);
}

uint64_t period_key(double p) {
  if (p == 0.0) p = 0.0;  // -0 and +0 compare equal
  uint64_t k;
  std::memcpy(&k, &p, sizeof k);
  return k;
}

}  // namespace

int srcrec_index(SrcRecTable* t) {
  const int n = t->npath();
  if (n < 1) return ST_BAD_ARG;
  if (t->weight.size() != (size_t)n) t->weight.assign(n, 1.0);
  // get_periods (src/src_rec.f90:126-156): distinct values, ascending
  std::unordered_map<uint64_t, int> pmap;
  std::vector<double> uniq;
  for (int i = 0; i < n; ++i) {
    const double p = t->period[i];
    if (std::isnan(p)) return ST_BAD_ARG;  // never equal to itself: no period
    if (pmap.emplace(period_key(p), (int)uniq.size()).second) uniq.push_back(p == 0.0 ? 0.0 : p);
  }
  t->periods = uniq;
  std::sort(t->periods.begin(), t->periods.end());
  for (int q = 0; q < (int)t->periods.size(); ++q) pmap[period_key(t->periods[q])] = q;
  t->per_id.resize(n);
  for (int i = 0; i < n; ++i) t->per_id[i] = pmap[period_key(t->period[i])];
  // get_sta (:178-226): station names in order of first appearance with
  // their first coordinates, then event names that are not stations
  std::unordered_map<std::string, int> smap;
  t->sta_name.clear();
  t->sta_lo.clear();
  t->sta_la.clear();
  auto add = [&](const std::string& name, double lo, double la) {
    const std::string k = rstrip(name);
    auto it = smap.find(k);
    if (it != smap.end()) return it->second;
    const int id = (int)t->sta_name.size();
    smap.emplace(k, id);
    t->sta_name.push_back(k);
    t->sta_lo.push_back(lo);
    t->sta_la.push_back(la);
    return id;
  };
  t->sta_id.resize(n);
  t->evt_id.resize(n);
  for (int i = 0; i < n; ++i) t->sta_id[i] = add(t->staname[i], t->stlo[i], t->stla[i]);
  for (int i = 0; i < n; ++i) t->evt_id[i] = add(t->evtname[i], t->evlo[i], t->evla[i]);
  t->built = false;
  return ST_OK;
}

// ---------------------------------------------------------------------------
// Work-list kernels.
// ---------------------------------------------------------------------------
namespace {

constexpr int kIntMax = 0x7fffffff;

__global__ void k_wl_init(long long n, int* first, int* cnt) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    first[k] = kIntMax;
    cnt[k] = 0;
  }
}

// Per path: the first path and the number of paths of its (event, period).
__global__ void k_wl_count(WorklistArgs A, int* first, int* cnt, int* slot) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.npath) return;
  const int p = A.per[i];
  if (A.pz[p]) {
    slot[i] = -1;
    return;
  }
  const long long key = (long long)A.evt[i] * A.P + p;
  atomicMin(first + key, i);
  slot[i] = atomicAdd(cnt + key, 1);
}

// Exclusive scan over a 1024-thread block; every thread calls it.
__device__ int block_exclusive_scan(int v, int* total) {
  __shared__ int ws[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = lane < nw ? ws[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    ws[lane] = w;
  }
  __syncthreads();
  const int pre = (wid > 0 ? ws[wid - 1] : 0) + x - v;
  *total = ws[nw - 1];
  __syncthreads();
  return pre;
}

// One block of 1024 threads: solves in station order, each event's periods
// in order of their first path (scatter_src_gather, src/src_rec.f90:338-369
// with get_periods_by_src :158-176), then the receiver offsets.
__global__ void __launch_bounds__(1024) k_wl_solves(WorklistArgs A, const int* first,
                                                    const int* cnt, int* sok, int* ebase) {
  const int S = A.S, P = A.P;
  int carry = 0, tot = 0;
  for (int e0 = 0; e0 < S; e0 += blockDim.x) {
    const int e = e0 + threadIdx.x;
    int ne = 0;
    if (e < S)
      for (int p = 0; p < P; ++p) ne += cnt[(long long)e * P + p] > 0;
    const int pre = block_exclusive_scan(ne, &tot);
    if (e < S) ebase[e] = carry + pre;
    carry += tot;
  }
  const int nsolve = carry;
  __syncthreads();
  for (long long key = threadIdx.x; key < (long long)S * P; key += blockDim.x) {
    const int c = cnt[key];
    if (c <= 0) continue;
    const int e = (int)(key / P), p = (int)(key - (long long)e * P);
    const int f = first[key];
    int rank = 0;
    for (int q = 0; q < P; ++q) {
      const long long k2 = (long long)e * P + q;
      rank += (cnt[k2] > 0 && first[k2] < f);
    }
    const int s = ebase[e] + rank;
    sok[key] = s;
    A.pidx[s] = p;
    A.wsta[s] = e;
    A.nrec[s] = c;
    A.srcx[s] = A.sta_lo[e];  // get_sta_pos (:327-336)
    A.srcy[s] = A.sta_la[e];
  }
  __syncthreads();
  carry = 0;
  for (int s0 = 0; s0 < nsolve; s0 += blockDim.x) {
    const int s = s0 + threadIdx.x;
    const int v = s < nsolve ? A.nrec[s] : 0;
    const int pre = block_exclusive_scan(v, &tot);
    if (s < nsolve) A.rec_off[s] = carry + pre;
    carry += tot;
  }
  if (threadIdx.x == 0) *A.d_nsolve = nsolve;
}

__global__ void k_wl_scatter(WorklistArgs A, const int* sok, const int* slot) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.npath || slot[i] < 0) return;
  const long long key = (long long)A.evt[i] * A.P + A.per[i];
  const int s = sok[key];
  A.recs[A.rec_off[s] + slot[i]] = i;
}

// One block per solve: its receivers sorted by path index (the order of
// get_evt_gather, :252-283) by ranking each against the whole segment,
// with their station's coordinates, time and weight.
__global__ void __launch_bounds__(128) k_wl_gather(WorklistArgs A) {
  __shared__ int tile[1024];
  const int s = blockIdx.x;
  if (s >= *A.d_nsolve) return;  // uniform over the block
  const int base = A.rec_off[s], n = A.nrec[s];
  for (int e0 = 0; e0 < n; e0 += blockDim.x) {
    const bool mine = e0 + (int)threadIdx.x < n;
    const int x = mine ? A.recs[base + e0 + threadIdx.x] : kIntMax;
    int rank = 0;
    for (int t0 = 0; t0 < n; t0 += 1024) {
      const int m = min(1024, n - t0);
      __syncthreads();
      for (int q = threadIdx.x; q < m; q += blockDim.x) tile[q] = A.recs[base + t0 + q];
      __syncthreads();
      for (int q = 0; q < m; ++q) rank += tile[q] < x;
    }
    if (mine) {
      const int pos = base + rank;
      const int st = A.sta[x];
      A.rpath[pos] = x;
      A.recx[pos] = A.sta_lo[st];
      A.recy[pos] = A.sta_la[st];
      A.rtt[pos] = A.tt[x];
      A.rweight[pos] = A.weight[x];
    }
  }
}

}  // namespace

void launch_worklist(const WorklistArgs& A, cudaStream_t st) {
  const long long SP = (long long)A.S * A.P;
  int* first = A.scratch;
  int* cnt = first + SP;
  int* sok = cnt + SP;
  int* slot = sok + SP;
  int* ebase = slot + A.npath;
  k_wl_init<<<(unsigned)std::min<long long>((SP + 255) / 256, 4096), 256, 0, st>>>(SP, first,
                                                                                   cnt);
  const unsigned gp = (unsigned)((A.npath + 255) / 256);
  k_wl_count<<<gp, 256, 0, st>>>(A, first, cnt, slot);
  k_wl_solves<<<1, 1024, 0, st>>>(A, first, cnt, sok, ebase);
  k_wl_scatter<<<gp, 256, 0, st>>>(A, sok, slot);
  const long long maxsolve = std::min<long long>(SP, A.npath);
  k_wl_gather<<<(unsigned)std::max<long long>(maxsolve, 1), 128, 0, st>>>(A);
}

}  // namespace sgb
