// Pieces shared by the separable level-step kernels (one step per launch in
// gm_level.cu, many steps per launch in gm_persist.cu).
#pragma once
#include "gm_common.cuh"

namespace gm {

template <typename real, int N>
struct RegCol {  // a strip column passed by value (stays in registers across the call)
  real v[N];
};

// Top-surface flux of the strip's nodes: each lane evaluates the faces of
// elements (x, y0-1+i), i = 0..BYT, at their 2 x 2 Gauss points and the node
// sums are gathered from the lane to the left.  Called by every lane of the
// warp (shuffles); one call per warp and launch, kept out of line so that the
// unrolled plane loop stays small.
template <typename real, int BYT>
__device__ __noinline__ RegCol<real, BYT> sep_surface(const Props<real> P, real w2, int x, int nx, int y0, int ny,
                                                      const RegCol<real, BYT + 2> T0c) {
  constexpr unsigned FULL = 0xffffffffu;
  const real* T0 = T0c.v;
  RegCol<real, BYT> out;
  real* surf = out.v;
  const real PQ = (real)0.78867513459481288225, MQ = (real)0.21132486540518711775;  // (1 +- 1/sqrt3)/2
  real c00[BYT + 1], c10[BYT + 1], c01[BYT + 1], c11[BYT + 1];
#pragma unroll
  for (int i = 0; i <= BYT; ++i) {  // element (x, y0 - 1 + i): strip rows i, i+1
    const real t10 = __shfl_down_sync(FULL, T0[i], 1), t11 = __shfl_down_sync(FULL, T0[i + 1], 1);
    c00[i] = c10[i] = c01[i] = c11[i] = 0;
    const int ey = y0 - 1 + i;
    if (x >= 0 && x < nx - 1 && ey >= 0 && ey < ny - 1) {
      const real t00 = T0[i], t01 = T0[i + 1];
#pragma unroll
      for (int qy = 0; qy < 2; ++qy)
#pragma unroll
        for (int qx = 0; qx < 2; ++qx) {
          const real px0 = qx ? MQ : PQ, px1 = qx ? PQ : MQ;
          const real py0 = qy ? MQ : PQ, py1 = qy ? PQ : MQ;
          const real w00 = rmul(px0, py0), w10 = rmul(px1, py0), w01 = rmul(px0, py1), w11 = rmul(px1, py1);
          const real Tq4 = rfma(w11, t11, rfma(w01, t01, rfma(w10, t10, rmul(w00, t00))));
          const real q = rmul(surface_flux(P, Tq4), w2);
          c00[i] = rfma(w00, q, c00[i]);
          c10[i] = rfma(w10, q, c10[i]);
          c01[i] = rfma(w01, q, c01[i]);
          c11[i] = rfma(w11, q, c11[i]);
        }
    }
  }
  // node row r: elements i = r (upper-y corners) and i = r + 1 (lower-y corners)
#pragma unroll
  for (int r = 0; r < BYT; ++r)
    surf[r] = radd(radd(c01[r], c00[r + 1]), __shfl_up_sync(FULL, radd(c11[r], c10[r + 1]), 1));
  return out;
}

}  // namespace gm
