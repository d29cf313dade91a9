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
// createPath.toolpath's.  The recurrences run on one thread (a call is a
// few hundred dependent FP64 additions); the rows are staged in shared
// memory and written out by the whole block.
#include <cuda_runtime.h>

#include "gm_common.cuh"

namespace gm {

constexpr int RUN_FIELDS = 11;  // kind, count, x, y, z, jump, ux, uy, dt, P, short

constexpr int ROWS_CHUNK = 128;  // rows staged in shared memory between the serial and the parallel part

// Thread 0 walks the run table serially (the FP64 recurrences), keeping the
// current run's fields in registers and staging a chunk of rows in shared
// memory; the whole block then writes the chunk out coalesced.
__global__ void __launch_bounds__(128) toolpath_rows_kernel(const double* __restrict__ runs, int nruns,
                                                            gm_toolpath_state* st, int nrows, int ngroups,
                                                            double* __restrict__ rows, double* __restrict__ dts) {
  __shared__ double srow[ROWS_CHUNK * 7];
  __shared__ double s_carry[8];  // x, y, t, tot, grp; run, k as doubles (exact below 2^53)
  if (threadIdx.x == 0) {
    s_carry[0] = st->x;
    s_carry[1] = st->y;
    s_carry[2] = st->t;
    s_carry[3] = 0.0;
    s_carry[4] = 0.0;
    s_carry[5] = (double)st->run;
    s_carry[6] = (double)st->k;
  }
  const int per = nrows / ngroups;
  for (int c0 = 0; c0 < nrows; c0 += ROWS_CHUNK) {
    const int cn = min(ROWS_CHUNK, nrows - c0);
    if (threadIdx.x == 0) {
      double x = s_carry[0], y = s_carry[1], t = s_carry[2], tot = s_carry[3], grp = s_carry[4];
      long long run = (long long)s_carry[5], k = (long long)s_carry[6];
      // fields of the current run, reloaded when the run changes
      long long loaded = -1, n = 0, nrun = 0;
      bool move = false;
      double r2 = 0, r3 = 0, r4 = 0, r5 = 0, r6 = 0, r7 = 0, r8 = 0, r9 = 0, r10 = 0;
      for (int i = 0; i < cn; ++i) {
        double v[7] = {0, 0, 0, 0, 0, 0, 0};
        while (run < nruns) {
          if (loaded != run) {
            const double* r = runs + run * RUN_FIELDS;
            n = (long long)r[1];
            move = r[0] == 0.0;
            r2 = r[2], r3 = r[3], r4 = r[4], r5 = r[5], r6 = r[6], r7 = r[7], r8 = r[8], r9 = r[9], r10 = r[10];
            nrun = n + ((move && r10 > 0.0) ? 1 : 0);
            loaded = run;
          }
          if (k < nrun) break;
          ++run;
          k = 0;
        }
        if (run < nruns) {
          if (move) {
            if (k == 0) {
              x = r2;
              y = r3;
            }
            const double d = k < n ? r8 : r10;
            x = __dadd_rn(x, __dmul_rn(r6, d));
            y = __dadd_rn(y, __dmul_rn(r7, d));
            v[0] = x;
            v[1] = y;
            v[4] = 1.0;
            v[5] = d;
            v[6] = r9;
          } else {
            v[0] = r2;
            v[1] = r3;
            v[5] = r8;
          }
          v[2] = r4;
          v[3] = r5;
          ++k;
        }
        for (int c = 0; c < 7; ++c) srow[7 * i + c] = v[c];
        t = __dadd_rn(t, v[5]);
        tot = __dadd_rn(tot, v[5]);
        grp = __dadd_rn(grp, v[5]);
        if ((c0 + i + 1) % per == 0) {
          dts[1 + (c0 + i) / per] = grp;
          grp = 0.0;
        }
      }
      s_carry[0] = x;
      s_carry[1] = y;
      s_carry[2] = t;
      s_carry[3] = tot;
      s_carry[4] = grp;
      s_carry[5] = (double)run;
      s_carry[6] = (double)k;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < 7 * cn; j += blockDim.x) rows[7LL * c0 + j] = srow[j];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    dts[0] = s_carry[3];
    st->run = (long long)s_carry[5];
    st->k = (long long)s_carry[6];
    st->x = s_carry[0];
    st->y = s_carry[1];
    st->t = s_carry[2];
    st->row += nrows;
  }
}

}  // namespace gm

extern "C" int gm_toolpath_rows(const double* runs, int nruns, gm_toolpath_state* state, int nrows, int ngroups,
                                double* rows, double* dts, void* stream) {
  if (!runs || nruns < 1 || !state || nrows < 1 || ngroups < 1 || nrows % ngroups || !rows || !dts)
    return GM_ERR_ARG;
  gm::toolpath_rows_kernel<<<1, 128, 0, (cudaStream_t)stream>>>(runs, nruns, state, nrows, ngroups, rows, dts);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}
