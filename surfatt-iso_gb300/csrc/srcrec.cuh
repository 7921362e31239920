// srcrec.cuh -- the src_rec table and the work list derived from it.
//
// SurfATT reads one row per path (travel time, station, event, period,
// weight) and derives, with string comparisons and a linear scan per
// (source, period) solve (src/src_rec.f90:126-369, src/measadj.f90:39-53):
//   periods   the distinct periods, ascending;
//   stations  the distinct station names in order of first appearance with
//             their first coordinates, then the event names that are not
//             stations, with the event coordinates;
//   solves    for every station in that order that is some path's event,
//             its periods in order of first appearance: (period, station);
//   receivers for each solve, the paths of that event and period in path
//             order, with the coordinates of their station.
// Here the host maps names and periods to integer ids once (hash maps), and
// the grouping runs on the GPU (srcrec.cu): a per-(event, period) count and
// first path, the solve order per event, a scatter of paths into their
// solve's segment, and a sort of every segment by path index.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace sgb {

struct SrcRecTable {
  // per path (the CSV's rows)
  std::vector<std::string> staname, evtname;
  std::vector<double> tt, stla, stlo, evla, evlo, period, weight, dist, vel;
  std::vector<std::string> header;  // input header without stel / evel, in file order
  bool has_weight = false, has_dist = false, has_vel = false;
  // derived on the host
  std::vector<double> periods;       // distinct, ascending
  std::vector<std::string> sta_name;  // station table
  std::vector<double> sta_lo, sta_la;
  std::vector<int> evt_id, sta_id, per_id;  // per path
  // work list (GPU-built)
  bool built = false;
  int nsolve = 0, nrec_total = 0;
  std::vector<int> pidx, sta, rec_off, nrec, rpath;
  std::vector<double> srcx, srcy, recx, recy, rtt, rweight;
  float build_ms = 0.f;
  int npath() const { return (int)tt.size(); }
};

// Ids of names and periods (the derived arrays above).  Returns 0 or 2
// (empty table, a period that is not a number).
int srcrec_index(SrcRecTable* t);

// Device work list of an indexed table.  evt / per / sta: per-path ids;
// pz[p] != 0 marks a period that gets no solve (exactly 0: the reference's
// get_periods_by_src skips it).  Buffers are device pointers; `scratch`
// holds 3*S*P + npath + S ints (S stations, P periods).  Writes nsolve to
// *d_nsolve.  Launches 5 kernels on st.
struct WorklistArgs {
  int npath, S, P;
  const int *evt, *per, *sta;
  const unsigned char* pz;
  const double *sta_lo, *sta_la, *tt, *weight;
  int* scratch;
  int* d_nsolve;
  int *pidx, *wsta, *rec_off, *nrec;
  double *srcx, *srcy;
  int* recs;  // npath, unsorted segments
  int* rpath;
  double *recx, *recy, *rtt, *rweight;
};
void launch_worklist(const WorklistArgs& A, cudaStream_t st);

}  // namespace sgb
