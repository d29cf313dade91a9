// Toolpath rows generated on the device in FP64.
//
// The reference writes the laser path as text, one row per fine time step,
// accumulating the position in host float64 (go_melt/createPath.py:126-160:
// x += vx * dt per step, a short remainder step, wait and dwell rows at a
// layer change), and the driver advances its time by the rows' dt
// (go_melt/go_melt.py:140-160, 467).  Here the host compiles the G-code into
// a short table of runs (createPath.toolpath_runs) and this kernel expands it
// chunk by chunk, carrying the run cursor, the position and the elapsed time
// in a device-resident FP64 state from call to call.  Products are rounded
// before the sums (__dmul_rn / __dadd_rn, never a fused multiply-add), as in
// the host's float64 arithmetic, so the rows are bit-identical to
// createPath.toolpath's.  One thread: a chunk is a few hundred dependent
// FP64 additions.
#include <cuda_runtime.h>

#include "gm_common.cuh"

namespace gm {

constexpr int RUN_FIELDS = 11;  // kind, count, x, y, z, jump, ux, uy, dt, P, short

__global__ void toolpath_rows_kernel(const double* __restrict__ runs, int nruns, gm_toolpath_state* st, int nrows,
                                     int ngroups, double* __restrict__ rows, double* __restrict__ dts) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  long long run = st->run, k = st->k;
  double x = st->x, y = st->y, t = st->t;
  const int per = nrows / ngroups;
  double tot = 0.0, grp = 0.0;
  for (int i = 0; i < nrows; ++i) {
    double v[7] = {0, 0, 0, 0, 0, 0, 0};
    bool have = false;
    while (run < nruns && !have) {
      const double* r = runs + run * RUN_FIELDS;
      const long long n = (long long)r[1];
      const bool move = r[0] == 0.0;
      const long long nrun = n + ((move && r[10] > 0.0) ? 1 : 0);
      if (k >= nrun) {
        ++run;
        k = 0;
        continue;
      }
      if (move) {
        if (k == 0) {
          x = r[2];
          y = r[3];
        }
        const double d = k < n ? r[8] : r[10];
        x = __dadd_rn(x, __dmul_rn(r[6], d));
        y = __dadd_rn(y, __dmul_rn(r[7], d));
        v[0] = x;
        v[1] = y;
        v[4] = 1.0;
        v[5] = d;
        v[6] = r[9];
      } else {
        v[0] = r[2];
        v[1] = r[3];
        v[5] = r[8];
      }
      v[2] = r[4];
      v[3] = r[5];
      ++k;
      have = true;
    }
    for (int c = 0; c < 7; ++c) rows[7LL * i + c] = v[c];
    t = __dadd_rn(t, v[5]);
    tot = __dadd_rn(tot, v[5]);
    grp = __dadd_rn(grp, v[5]);
    if ((i + 1) % per == 0) {
      dts[1 + i / per] = grp;
      grp = 0.0;
    }
  }
  dts[0] = tot;
  st->run = run;
  st->k = k;
  st->x = x;
  st->y = y;
  st->t = t;
  st->row += nrows;
}

}  // namespace gm

extern "C" int gm_toolpath_rows(const double* runs, int nruns, gm_toolpath_state* state, int nrows, int ngroups,
                                double* rows, double* dts, void* stream) {
  if (!runs || nruns < 1 || !state || nrows < 1 || ngroups < 1 || nrows % ngroups || !rows || !dts)
    return GM_ERR_ARG;
  gm::toolpath_rows_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(runs, nruns, state, nrows, ngroups, rows, dts);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}
