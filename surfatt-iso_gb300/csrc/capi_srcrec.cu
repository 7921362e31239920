// capi_srcrec.cu -- C ABI of the src_rec table: CSV reading and writing
// (src/shared/src_rec_parser.f90:20-64, src/src_rec.f90:285-325), the
// station / period tables and the GPU-built work list (srcrec.cu).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "../../include/surfatt_gb300.h"
#include "common.cuh"
#include "host_buf.cuh"
#include "srcrec.cuh"

using namespace sgb;

struct surfatt_srcrec {
  SrcRecTable t;
};

namespace {

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && (s[a] == ' ' || s[a] == '\t' || s[a] == '\r' || s[a] == '\n')) ++a;
  while (b > a && (s[b - 1] == ' ' || s[b - 1] == '\t' || s[b - 1] == '\r' || s[b - 1] == '\n'))
    --b;
  if (b - a >= 2 && ((s[a] == '"' && s[b - 1] == '"') || (s[a] == '\'' && s[b - 1] == '\''))) {
    ++a;
    --b;
  }
  return s.substr(a, b - a);
}

std::vector<std::string> split(const std::string& line) {
  std::vector<std::string> out;
  std::string cur;
  bool quoted = false;
  for (char ch : line) {
    if (ch == '"') quoted = !quoted;
    if (ch == ',' && !quoted) {
      out.push_back(trim(cur));
      cur.clear();
    } else {
      cur += ch;
    }
  }
  out.push_back(trim(cur));
  return out;
}

bool to_double(const std::string& s, double* v) {
  if (s.empty()) return false;
  char* end = nullptr;
  *v = std::strtod(s.c_str(), &end);
  // Fortran reads a D exponent as E
  if (end && *end && (*end == 'd' || *end == 'D')) {
    std::string t = s;
    t[end - s.c_str()] = 'e';
    *v = std::strtod(t.c_str(), &end);
    return end && *end == 0;
  }
  return end && *end == 0;
}

// gps2dist_scalar (src/shared/utils.f90:1250-1262) with the constants of
// src/shared/shared_par.f90:11-13.
double gps2dist(double lat0, double lon0, double lat1, double lon1) {
  const double deg2rad = PI_S / 180.0;
  const double dlat = (lat0 - lat1) * deg2rad, dlon = (lon1 - lon0) * deg2rad;
  const double s1 = std::sin(dlat * 0.5), s2 = std::sin(dlon * 0.5);
  const double a = s1 * s1 + s2 * s2 * std::cos(lat0 * deg2rad) * std::cos(lat1 * deg2rad);
  return 6371.0 * (2.0 * std::atan2(std::sqrt(a), std::sqrt(1.0 - a)));
}

// A Fortran Fw.d edit of v without its leading blanks (the CSV writer
// left-adjusts and trims, src/src_rec.f90:313-323); w = 0 is the minimal
// width; a value wider than w prints as w asterisks.
std::string fortran_f(double v, int w, int d) {
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.*f", d, v);
  std::string s(buf);
  if (w > 0 && (int)s.size() > w) return std::string(w, '*');
  return s;
}

int index_or(SrcRecTable& t) { return srcrec_index(&t); }

}  // namespace

extern "C" {

surfatt_status_t surfatt_srcrec_read_csv(const char* fname, surfatt_srcrec_t** out) {
  if (!fname || !out) return SURFATT_BAD_ARG;
  *out = nullptr;
  std::ifstream f(fname);
  if (!f) return SURFATT_BAD_ARG;  // the reference prints "No such file" and stops
  std::string line;
  if (!std::getline(f, line)) return SURFATT_BAD_ARG;
  std::vector<std::string> hdr = split(line);
  auto col = [&](const char* name) {
    int idx = -1;
    for (int i = 0; i < (int)hdr.size(); ++i)
      if (hdr[i] == name) idx = i;  // the last match, as col_index
    return idx;
  };
  const int c_tt = col("tt"), c_sn = col("staname"), c_sla = col("stla"), c_slo = col("stlo");
  const int c_en = col("evtname"), c_ela = col("evla"), c_elo = col("evlo"), c_p = col("period");
  const int c_w = col("weight"), c_d = col("dist"), c_v = col("vel");
  if (c_tt < 0 || c_sn < 0 || c_sla < 0 || c_slo < 0 || c_en < 0 || c_ela < 0 || c_elo < 0 ||
      c_p < 0)
    return SURFATT_BAD_ARG;  // "Column ... not found in the header"
  auto* h = new surfatt_srcrec();
  SrcRecTable& t = h->t;
  for (const auto& name : hdr)
    if (name != "stel" && name != "evel") t.header.push_back(name);
  t.has_weight = c_w >= 0;
  t.has_dist = c_d >= 0;
  t.has_vel = c_v >= 0;
  while (std::getline(f, line)) {
    if (trim(line).empty()) continue;
    const std::vector<std::string> v = split(line);
    if (v.size() < hdr.size()) {
      delete h;
      return SURFATT_BAD_ARG;
    }
    double x[11];
    const int cols[8] = {c_tt, c_sla, c_slo, c_ela, c_elo, c_p, c_w, c_d};
    bool ok = true;
    for (int k = 0; k < 6; ++k) ok = ok && to_double(v[cols[k]], &x[k]);
    if (t.has_weight) ok = ok && to_double(v[c_w], &x[6]);
    if (t.has_dist) ok = ok && to_double(v[c_d], &x[7]);
    if (t.has_vel) ok = ok && to_double(v[c_v], &x[8]);
    if (!ok) {
      delete h;
      return SURFATT_BAD_ARG;
    }
    t.tt.push_back(x[0]);
    t.stla.push_back(x[1]);
    t.stlo.push_back(x[2]);
    t.evla.push_back(x[3]);
    t.evlo.push_back(x[4]);
    t.period.push_back(x[5]);
    t.staname.push_back(v[c_sn]);
    t.evtname.push_back(v[c_en]);
    t.weight.push_back(t.has_weight ? x[6] : 1.0);  // src_rec_parser.f90:45-49
    t.dist.push_back(t.has_dist ? x[7] : gps2dist(x[1], x[2], x[3], x[4]));  // :50-57
    t.vel.push_back(t.has_vel ? x[8] : t.dist.back() / x[0]);                 // :58-62
  }
  if (index_or(t) != ST_OK) {
    delete h;
    return SURFATT_BAD_ARG;
  }
  *out = h;
  return SURFATT_OK;
}

surfatt_status_t surfatt_srcrec_create(int npath, const char* const* evtname,
                                       const char* const* staname, const double* stla,
                                       const double* stlo, const double* evla,
                                       const double* evlo, const double* period,
                                       const double* tt, const double* weight,
                                       surfatt_srcrec_t** out) {
  if (!out || npath < 1 || !evtname || !staname || !stla || !stlo || !evla || !evlo || !period ||
      !tt)
    return SURFATT_BAD_ARG;
  *out = nullptr;
  auto* h = new surfatt_srcrec();
  SrcRecTable& t = h->t;
  t.has_weight = weight != nullptr;
  for (int i = 0; i < npath; ++i) {
    if (!evtname[i] || !staname[i]) {
      delete h;
      return SURFATT_BAD_ARG;
    }
    t.evtname.emplace_back(evtname[i]);
    t.staname.emplace_back(staname[i]);
    t.stla.push_back(stla[i]);
    t.stlo.push_back(stlo[i]);
    t.evla.push_back(evla[i]);
    t.evlo.push_back(evlo[i]);
    t.period.push_back(period[i]);
    t.tt.push_back(tt[i]);
    t.weight.push_back(weight ? weight[i] : 1.0);
    t.dist.push_back(gps2dist(stla[i], stlo[i], evla[i], evlo[i]));
    t.vel.push_back(t.dist.back() / tt[i]);
  }
  if (index_or(t) != ST_OK) {
    delete h;
    return SURFATT_BAD_ARG;
  }
  *out = h;
  return SURFATT_OK;
}

void surfatt_srcrec_destroy(surfatt_srcrec_t* h) { delete h; }

surfatt_status_t surfatt_srcrec_info(const surfatt_srcrec_t* h, int* npath, int* nperiod,
                                     int* nsta, int* nsolve) {
  if (!h) return SURFATT_BAD_ARG;
  if (npath) *npath = h->t.npath();
  if (nperiod) *nperiod = (int)h->t.periods.size();
  if (nsta) *nsta = (int)h->t.sta_name.size();
  if (nsolve) *nsolve = h->t.built ? h->t.nsolve : -1;
  return SURFATT_OK;
}

surfatt_status_t surfatt_srcrec_periods(const surfatt_srcrec_t* h, double* periods) {
  if (!h || !periods) return SURFATT_BAD_ARG;
  std::copy(h->t.periods.begin(), h->t.periods.end(), periods);
  return SURFATT_OK;
}

surfatt_status_t surfatt_srcrec_stations(const surfatt_srcrec_t* h, double* stlo, double* stla) {
  if (!h) return SURFATT_BAD_ARG;
  if (stlo) std::copy(h->t.sta_lo.begin(), h->t.sta_lo.end(), stlo);
  if (stla) std::copy(h->t.sta_la.begin(), h->t.sta_la.end(), stla);
  return SURFATT_OK;
}

const char* surfatt_srcrec_station_name(const surfatt_srcrec_t* h, int i) {
  if (!h || i < 0 || i >= (int)h->t.sta_name.size()) return nullptr;
  return h->t.sta_name[i].c_str();
}

surfatt_status_t surfatt_srcrec_paths(const surfatt_srcrec_t* h, double* tt, double* weight,
                                      double* period, int* evt_station, int* station,
                                      int* period_index) {
  if (!h) return SURFATT_BAD_ARG;
  const SrcRecTable& t = h->t;
  if (tt) std::copy(t.tt.begin(), t.tt.end(), tt);
  if (weight) std::copy(t.weight.begin(), t.weight.end(), weight);
  if (period) std::copy(t.period.begin(), t.period.end(), period);
  if (evt_station) std::copy(t.evt_id.begin(), t.evt_id.end(), evt_station);
  if (station) std::copy(t.sta_id.begin(), t.sta_id.end(), station);
  if (period_index) std::copy(t.per_id.begin(), t.per_id.end(), period_index);
  return SURFATT_OK;
}

surfatt_status_t surfatt_srcrec_build_worklist(surfatt_srcrec_t* h, int device, int* nsolve) {
  if (!h) return SURFATT_BAD_ARG;
  SrcRecTable& t = h->t;
  const int n = t.npath(), S = (int)t.sta_name.size(), P = (int)t.periods.size();
  CK(cudaSetDevice(device));
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    cudaGetLastError();
    return SURFATT_CUDA_ERROR;
  }
  std::vector<unsigned char> pz(P);
  for (int p = 0; p < P; ++p) pz[p] = t.periods[p] == 0.0;
  const size_t SP = (size_t)S * P, nI = sizeof(int), nD = sizeof(double);
  DBuf b_evt, b_per, b_sta, b_pz, b_lo, b_la, b_tt, b_w, b_scr, b_ns, b_pidx, b_wsta, b_off,
      b_nrec, b_sx, b_sy, b_recs, b_rpath, b_rx, b_ry, b_rtt, b_rw;
  DBuf* all[] = {&b_evt, &b_per, &b_sta, &b_pz,  &b_lo,  &b_la,   &b_tt, &b_w,
                 &b_scr, &b_ns,  &b_pidx, &b_wsta, &b_off, &b_nrec, &b_sx, &b_sy,
                 &b_recs, &b_rpath, &b_rx, &b_ry, &b_rtt, &b_rw};
  const size_t maxs = std::min<size_t>(SP, (size_t)n);
  int r = 0;
  r |= b_evt.ensure(n * nI) | b_per.ensure(n * nI) | b_sta.ensure(n * nI) | b_pz.ensure(P);
  r |= b_lo.ensure(S * nD) | b_la.ensure(S * nD) | b_tt.ensure(n * nD) | b_w.ensure(n * nD);
  r |= b_scr.ensure((3 * SP + n + S) * nI) | b_ns.ensure(nI);
  r |= b_pidx.ensure(maxs * nI) | b_wsta.ensure(maxs * nI) | b_off.ensure(maxs * nI) |
       b_nrec.ensure(maxs * nI) | b_sx.ensure(maxs * nD) | b_sy.ensure(maxs * nD);
  r |= b_recs.ensure(n * nI) | b_rpath.ensure(n * nI) | b_rx.ensure(n * nD) |
       b_ry.ensure(n * nD) | b_rtt.ensure(n * nD) | b_rw.ensure(n * nD);
  auto cleanup = [&]() {
    for (DBuf* b : all) b->release();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
  };
  if (r) {
    cleanup();
    return SURFATT_OOM;
  }
  cudaMemcpyAsync(b_evt.p, t.evt_id.data(), n * nI, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(b_per.p, t.per_id.data(), n * nI, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(b_sta.p, t.sta_id.data(), n * nI, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(b_pz.p, pz.data(), P, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(b_lo.p, t.sta_lo.data(), S * nD, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(b_la.p, t.sta_la.data(), S * nD, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(b_tt.p, t.tt.data(), n * nD, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(b_w.p, t.weight.data(), n * nD, cudaMemcpyHostToDevice, st);
  WorklistArgs A{n,
                 S,
                 P,
                 b_evt.as<int>(),
                 b_per.as<int>(),
                 b_sta.as<int>(),
                 b_pz.as<unsigned char>(),
                 b_lo.as<double>(),
                 b_la.as<double>(),
                 b_tt.as<double>(),
                 b_w.as<double>(),
                 b_scr.as<int>(),
                 b_ns.as<int>(),
                 b_pidx.as<int>(),
                 b_wsta.as<int>(),
                 b_off.as<int>(),
                 b_nrec.as<int>(),
                 b_sx.as<double>(),
                 b_sy.as<double>(),
                 b_recs.as<int>(),
                 b_rpath.as<int>(),
                 b_rx.as<double>(),
                 b_ry.as<double>(),
                 b_rtt.as<double>(),
                 b_rw.as<double>()};
  cudaEventRecord(e0, st);
  launch_worklist(A, st);
  cudaEventRecord(e1, st);
  int ns = 0;
  cudaMemcpyAsync(&ns, b_ns.p, nI, cudaMemcpyDeviceToHost, st);
  cudaError_t err = cudaStreamSynchronize(st);
  if (err == cudaSuccess) err = cudaGetLastError();
  if (err != cudaSuccess) {
    std::fprintf(stderr, "surfatt_gb300: work-list build failed: %s\n", cudaGetErrorString(err));
    cleanup();
    return SURFATT_CUDA_ERROR;
  }
  cudaEventElapsedTime(&t.build_ms, e0, e1);
  int nr = 0;
  t.pidx.resize(ns);
  t.sta.resize(ns);
  t.rec_off.resize(ns);
  t.nrec.resize(ns);
  t.srcx.resize(ns);
  t.srcy.resize(ns);
  cudaMemcpy(t.pidx.data(), b_pidx.p, ns * nI, cudaMemcpyDeviceToHost);
  cudaMemcpy(t.sta.data(), b_wsta.p, ns * nI, cudaMemcpyDeviceToHost);
  cudaMemcpy(t.rec_off.data(), b_off.p, ns * nI, cudaMemcpyDeviceToHost);
  cudaMemcpy(t.nrec.data(), b_nrec.p, ns * nI, cudaMemcpyDeviceToHost);
  cudaMemcpy(t.srcx.data(), b_sx.p, ns * nD, cudaMemcpyDeviceToHost);
  cudaMemcpy(t.srcy.data(), b_sy.p, ns * nD, cudaMemcpyDeviceToHost);
  if (ns > 0) nr = t.rec_off[ns - 1] + t.nrec[ns - 1];
  t.rpath.resize(nr);
  t.recx.resize(nr);
  t.recy.resize(nr);
  t.rtt.resize(nr);
  t.rweight.resize(nr);
  cudaMemcpy(t.rpath.data(), b_rpath.p, nr * nI, cudaMemcpyDeviceToHost);
  cudaMemcpy(t.recx.data(), b_rx.p, nr * nD, cudaMemcpyDeviceToHost);
  cudaMemcpy(t.recy.data(), b_ry.p, nr * nD, cudaMemcpyDeviceToHost);
  cudaMemcpy(t.rtt.data(), b_rtt.p, nr * nD, cudaMemcpyDeviceToHost);
  err = cudaMemcpy(t.rweight.data(), b_rw.p, nr * nD, cudaMemcpyDeviceToHost);
  cleanup();
  if (err != cudaSuccess) return SURFATT_CUDA_ERROR;
  t.nsolve = ns;
  t.nrec_total = nr;
  t.built = true;
  if (nsolve) *nsolve = ns;
  return SURFATT_OK;
}

surfatt_status_t surfatt_srcrec_worklist(const surfatt_srcrec_t* h, int* pidx, int* sta,
                                         double* srcx, double* srcy, int* rec_off, int* nrec,
                                         double* recx, double* recy, double* tt,
                                         double* weight, int* path) {
  if (!h || !h->t.built) return SURFATT_BAD_ARG;
  const SrcRecTable& t = h->t;
  auto cp = [](const auto& v, auto* out) {
    if (out) std::copy(v.begin(), v.end(), out);
  };
  cp(t.pidx, pidx);
  cp(t.sta, sta);
  cp(t.srcx, srcx);
  cp(t.srcy, srcy);
  cp(t.rec_off, rec_off);
  cp(t.nrec, nrec);
  cp(t.recx, recx);
  cp(t.recy, recy);
  cp(t.rtt, tt);
  cp(t.rweight, weight);
  cp(t.rpath, path);
  return SURFATT_OK;
}

surfatt_status_t surfatt_srcrec_build_timing(const surfatt_srcrec_t* h, double* kernel_ms,
                                             int* launches) {
  if (!h || !h->t.built) return SURFATT_BAD_ARG;
  if (kernel_ms) *kernel_ms = h->t.build_ms;
  if (launches) *launches = 5;
  return SURFATT_OK;
}

surfatt_status_t surfatt_srcrec_write_csv(const surfatt_srcrec_t* h, const char* fname,
                                          const double* tt_fwd) {
  if (!h || !fname || !tt_fwd) return SURFATT_BAD_ARG;
  const SrcRecTable& t = h->t;
  FILE* f = std::fopen(fname, "w");
  if (!f) return SURFATT_BAD_ARG;  // the reference stops: 'Cannot open'
  std::fputs("tt,staname,stla,stlo,evtname,evla,evlo,period,weight,dist,vel\n", f);
  for (int i = 0; i < t.npath(); ++i) {
    const double d = t.dist[i];
    std::fprintf(f, "%s,%s,%s,%s,%s,%s,%s,%s,%s,%s,%s\n", fortran_f(tt_fwd[i], 0, 6).c_str(),
                 t.staname[i].c_str(), fortran_f(t.stla[i], 9, 4).c_str(),
                 fortran_f(t.stlo[i], 9, 4).c_str(), t.evtname[i].c_str(),
                 fortran_f(t.evla[i], 9, 4).c_str(), fortran_f(t.evlo[i], 9, 4).c_str(),
                 fortran_f(t.period[i], 0, 4).c_str(), fortran_f(t.weight[i], 6, 4).c_str(),
                 fortran_f(d, 12, 4).c_str(), fortran_f(d / tt_fwd[i], 10, 6).c_str());
  }
  return std::fclose(f) == 0 ? SURFATT_OK : SURFATT_BAD_ARG;
}

}  // extern "C"
