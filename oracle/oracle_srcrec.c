/*
 * oracle_srcrec.c -- CPU oracle (test infrastructure only) for the work
 * list and receiver gathers that SurfATT derives from its src_rec table.
 * Plain-C restatement, with the reference's string comparisons and linear
 * scans, of:
 *   src/src_rec.f90   get_periods          :126-156
 *                     get_periods_by_src   :158-176
 *                     get_sta              :178-226
 *                     get_evt_gather       :252-283
 *                     get_sta_pos          :327-336
 *                     scatter_src_gather   :338-369
 *   src/measadj.f90   get_recs             :39-53
 *
 * Names compare as Fortran character values (trailing blanks ignored);
 * periods compare exactly.  Kept on purpose: get_periods_by_src tests a
 * period against all nperiod slots of its zero-initialised list, so a
 * period of exactly 0 would be skipped (the reference's behaviour).
 * Outputs are 0-based.  Parity unpinned by the reference (no tests for
 * these routines, not buildable here); pinned by the test suite against
 * the example tables' structure and a Python restatement.
 */
#include <stdlib.h>
#include <string.h>

#include "surfatt_oracle.h"

/* Fortran character equality: equal after dropping trailing blanks. */
static int orc_name_eq(const char* a, const char* b) {
  size_t la = strlen(a), lb = strlen(b);
  while (la && a[la - 1] == ' ') --la;
  while (lb && b[lb - 1] == ' ') --lb;
  return la == lb && memcmp(a, b, la) == 0;
}

static int orc_cmp_double(const void* x, const void* y) {
  const double a = *(const double*)x, b = *(const double*)y;
  return a < b ? -1 : (a > b ? 1 : 0);
}

/* Capacities: periods npath, stations 2*npath (names are stored as
 * pointers into the inputs in sta_name), solves npath, receivers npath. */
int orc_srcrec_worklist(int npath, const char* const* evtname, const char* const* staname,
                        const double* stla, const double* stlo, const double* evla,
                        const double* evlo, const double* period, const double* tt,
                        const double* weight, int* nperiod_out, double* periods,
                        int* nsta_out, const char** sta_name, double* sta_lo, double* sta_la,
                        int* nsolve_out, int* pidx, int* sta, double* srcx, double* srcy,
                        int* rec_off, int* nrec, double* recx, double* recy, double* rtt,
                        double* rweight, int* rpath) {
  if (npath < 1) return 2;
  /* get_periods */
  int np = 1;
  periods[0] = period[0];
  for (int i = 1; i < npath; ++i) {
    int seen = 0;
    for (int q = 0; q < np; ++q) seen |= periods[q] == period[i];
    if (!seen) periods[np++] = period[i];
  }
  qsort(periods, np, sizeof(double), orc_cmp_double);
  *nperiod_out = np;
  /* get_sta: unique stanames (first coordinates), then unique evtnames */
  int ns = 0;
  for (int i = 0; i < npath; ++i) {
    int seen = 0;
    for (int q = 0; q < ns && !seen; ++q) seen = orc_name_eq(sta_name[q], staname[i]);
    if (!seen) {
      sta_name[ns] = staname[i];
      sta_la[ns] = stla[i];
      sta_lo[ns] = stlo[i];
      ++ns;
    }
  }
  for (int i = 0; i < npath; ++i) {
    int seen = 0;
    for (int q = 0; q < ns && !seen; ++q) seen = orc_name_eq(sta_name[q], evtname[i]);
    if (!seen) {
      sta_name[ns] = evtname[i];
      sta_la[ns] = evla[i];
      sta_lo[ns] = evlo[i];
      ++ns;
    }
  }
  *nsta_out = ns;
  /* scatter_src_gather: stations in order; per event its periods in
   * first-occurrence order (get_periods_by_src) */
  double* stp = (double*)malloc(np * sizeof(double));
  int nsolve = 0, nr_tot = 0;
  for (int j = 0; j < ns; ++j) {
    int is_evt = 0;
    for (int i = 0; i < npath && !is_evt; ++i) is_evt = orc_name_eq(evtname[i], sta_name[j]);
    if (!is_evt) continue;
    for (int q = 0; q < np; ++q) stp[q] = 0.0;
    int n = 0;
    for (int i = 0; i < npath; ++i) {
      if (!orc_name_eq(evtname[i], sta_name[j])) continue;
      int seen = 0;
      for (int q = 0; q < np; ++q) seen |= stp[q] == period[i];  /* all nperiod slots */
      if (seen) continue;
      stp[n++] = period[i];
      int ip = -1;  /* findloc(periods, period) */
      for (int q = 0; q < np && ip < 0; ++q)
        if (periods[q] == period[i]) ip = q;
      /* one solve (period ip, source j): get_recs */
      const int s = nsolve++;
      pidx[s] = ip;
      sta[s] = j;
      int k = -1; /* get_sta_pos: find_loc(staname, src_name) */
      for (int q = 0; q < ns && k < 0; ++q)
        if (orc_name_eq(sta_name[q], sta_name[j])) k = q;
      srcx[s] = sta_lo[k];
      srcy[s] = sta_la[k];
      rec_off[s] = nr_tot;
      int cnt = 0;
      for (int m = 0; m < npath; ++m) {  /* get_evt_gather */
        if (!(orc_name_eq(evtname[m], sta_name[j]) && period[m] == periods[ip])) continue;
        const int r = nr_tot + cnt++;
        rpath[r] = m;
        rtt[r] = tt[m];
        rweight[r] = weight ? weight[m] : 1.0;
        for (int q = 0; q < ns; ++q)  /* the last matching station, as written */
          if (orc_name_eq(sta_name[q], staname[m])) {
            recx[r] = sta_lo[q];
            recy[r] = sta_la[q];
          }
      }
      nrec[s] = cnt;
      nr_tot += cnt;
    }
  }
  free(stp);
  *nsolve_out = nsolve;
  return 0;
}
