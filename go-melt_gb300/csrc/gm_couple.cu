// Fine -> coarse coupling terms and the coarse laser source.
//
// Replaces the products of the reference's coarse-at-fine shape tables
// (computeCoarseFineShapeFunctions, go_melt/computeFunctions.py:1213-1358)
// with fine-level fields and their BCOO projection:
//   flux term  V_A -= sum_e sum_q grad Nc_A(q) . (kbar_e grad T'_e(q)) w
//              (computeL1TprimeTerms_Part1 :2733-2810,
//               computeL2TprimeTerms_Part1 :2857-2914,
//               computeCoarseTprimeTerm_jax :1477-1565)
//   mass term  V_A -= sum_e sum_q Nc_A(q) rcbar_e (T'a - T'b)_e(q) w / dt
//              (computeL1TprimeTerms_Part2 :3057-3132,
//               computeL2TprimeTerms_Part2 :3169-3221,
//               computeCoarseTprimeMassTerm_jax :1396-1474)
//   source     F_A += mean_p sum_e sum_q Nc_A(q) Q_p(q) w
//              (computeLevelSource :2667-2730, computeSources :928-988)
// with the reference's conventions: Nc and grad Nc are evaluated with the
// coarse element of each quadrature point, the result is assigned to the
// coarse nodes of quadrature point 0 of the fine element, k and rho*c enter
// as element means of nodal values.
//
// Everything is separable per axis: per fine element index and Gauss side the
// host supplies the two 1-D coarse weights (phi0, phi1), the coarse element of
// side 0, and per coarse element the range of fine elements assigned to it.
// One warp reduces one fine sub-box (at most 4x4x4 elements) of one coarse
// element to 8 partial sums; a gather kernel adds the partials of the up to 8
// coarse elements around each coarse node in a fixed order (deterministic,
// no atomics).  The source is a sum over laser positions of rank-1 tensors of
// 1-D factors, evaluated directly on the coarse node box.
#include <math.h>

#include "gm_common.cuh"

namespace gm {

constexpr int SB = 4;              // fine elements per sub-box edge
constexpr int SBN = (SB + 1) * (SB + 1) * (SB + 1);

template <typename real>
struct CoupleAxis {
  int nfe;
  const real* cw;    // [(e*2+s)*2 + A]
  const int* node0;  // [e]
  int cb_lo, ncb;
  const int* flo;
  const int* fhi;
  int nch;
  real invH;
};

template <typename real>
struct CoupleK {
  int fnx, fny;
  CoupleAxis<real> ax[3];
  const real* T;
  const uint8_t* ph;
  long long substrate;
  const real* k_arr;
  const real* rc_arr;
  const real* Tp;
  const real* dTa;
  const real* dTb;
  const double* dt;
  real wq;
  real cf[3];  // -2 wq / (H_d h_d): constant factor of the flux term along axis d
  int kconst;  // k and rho*c independent of phase and temperature: no per-node properties
  real* partials;
  long long nitems;
  int nchunk;
  Props<real> p;
};

template <typename real>
__device__ __forceinline__ real warp_sum(real v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// 2x2 Gauss-side transform of values d[b1][b2] given at the corners of a
// face: out[q1][q2] = sum_b psi[b1][q1] psi[b2][q2] d[b1][b2], psi the 1-D
// linear shape functions at the two Gauss points.
template <typename real>
__device__ __forceinline__ void psi2(const real d[2][2], real out[2][2]) {
  const real PQ = (real)0.78867513459481288225, MQ = (real)0.21132486540518711775;
  real u[2][2];  // u[q1][b2]
#pragma unroll
  for (int b2 = 0; b2 < 2; ++b2) {
    u[0][b2] = PQ * d[0][b2] + MQ * d[1][b2];
    u[1][b2] = MQ * d[0][b2] + PQ * d[1][b2];
  }
#pragma unroll
  for (int q1 = 0; q1 < 2; ++q1) {
    out[q1][0] = PQ * u[q1][0] + MQ * u[q1][1];
    out[q1][1] = MQ * u[q1][0] + PQ * u[q1][1];
  }
}

// Contraction with two 1-D coarse weight sets:
// out[A1][A2] = sum_q phA[A1][q1] phB[A2][q2] G[q1][q2].
template <typename real>
__device__ __forceinline__ void contract2(const real phA[2][2], const real phB[2][2], const real G[2][2],
                                          real out[2][2]) {
  real v[2][2];  // v[A1][q2]
#pragma unroll
  for (int A1 = 0; A1 < 2; ++A1)
#pragma unroll
    for (int q2 = 0; q2 < 2; ++q2) v[A1][q2] = phA[A1][0] * G[0][q2] + phA[A1][1] * G[1][q2];
#pragma unroll
  for (int A1 = 0; A1 < 2; ++A1)
#pragma unroll
    for (int A2 = 0; A2 < 2; ++A2) out[A1][A2] = phB[A2][0] * v[A1][0] + phB[A2][1] * v[A1][1];
}

// One warp per item = (coarse element, fine sub-box of at most 4x4x4
// elements).  The sub-box's nodes are staged once (T' or dT', k, rho*c) at
// fixed strides 1, 5, 25; each lane then handles up to two fine elements.
// All per-element products are sum-factorised along the axes.
template <typename real>
__global__ void __launch_bounds__(128) couple_kernel(const CoupleK<real> a) {
  pdl_begin();
  constexpr int S1 = SB + 1, S2 = S1 * S1;
  __shared__ V4<real> sR[4][SBN];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const real PQ = (real)0.78867513459481288225, MQ = (real)0.21132486540518711775;
  const bool flux = a.Tp != nullptr, mass = a.dTa != nullptr;
  const real wdt = mass ? a.wq / (real)(*a.dt) : (real)0;
  const int fnxy = a.fnx * a.fny;
  const long long nw = (long long)gridDim.x * 4;
  for (long long item = blockIdx.x * 4LL + warp; item < a.nitems; item += nw) {
    const int chunk = (int)(item % a.nchunk);
    long long ce = item / a.nchunk;
    const int cx = (int)(ce % a.ax[0].ncb);
    ce /= a.ax[0].ncb;
    const int cy = (int)(ce % a.ax[1].ncb);
    const int cz = (int)(ce / a.ax[1].ncb);
    const int kx = chunk % a.ax[0].nch, ky = (chunk / a.ax[0].nch) % a.ax[1].nch,
              kz = chunk / (a.ax[0].nch * a.ax[1].nch);
    const int e0x = a.ax[0].flo[cx] + kx * SB, e0y = a.ax[1].flo[cy] + ky * SB, e0z = a.ax[2].flo[cz] + kz * SB;
    const int nbx = min(a.ax[0].fhi[cx], e0x + SB) - e0x;
    const int nby = min(a.ax[1].fhi[cy], e0y + SB) - e0y;
    const int nbz = min(a.ax[2].fhi[cz], e0z + SB) - e0z;
    real acc[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) acc[i] = 0;
    if (nbx > 0 && nby > 0 && nbz > 0) {
      for (int i = lane; i < SBN; i += 32) {
        const int lx = i % S1, ly = (i / S1) % S1, lz = i / S2;
        if (lx <= nbx && ly <= nby && lz <= nbz) {
          const int id = (e0x + lx) + (e0y + ly) * a.fnx + (e0z + lz) * fnxy;
          real k = a.p.k_fluid, c = a.p.rho * a.p.cp_fluid;
          if (!a.kconst) node_props_sel(a.p, a.T[id], a.ph ? (uint32_t)a.ph[id] : 0u, id < a.substrate, k, c);
          if (a.k_arr) {
            k = a.k_arr[id];
            c = a.rc_arr[id];
          }
          V4<real> r;
          r.x = flux ? a.Tp[id] : (real)0;
          r.y = mass ? a.dTa[id] - a.dTb[id] : (real)0;
          r.z = k;
          r.w = c;
          sR[warp][i] = r;
        }
      }
      __syncwarp();
#pragma unroll
      for (int rr = 0; rr < 2; ++rr) {
        const int f = lane + 32 * rr;
        const int fx = f & 3, fy = (f >> 2) & 3, fz = f >> 4;
        if (fx >= nbx || fy >= nby || fz >= nbz) continue;
        const int ex = e0x + fx, ey = e0y + fy, ez = e0z + fz;
        real ph[3][2][2];  // ph[d][A][s]: 1-D coarse weight of local coarse node A at Gauss side s
#pragma unroll
        for (int s = 0; s < 2; ++s) {
          ph[0][0][s] = a.ax[0].cw[(ex * 2 + s) * 2 + 0];
          ph[0][1][s] = a.ax[0].cw[(ex * 2 + s) * 2 + 1];
          ph[1][0][s] = a.ax[1].cw[(ey * 2 + s) * 2 + 0];
          ph[1][1][s] = a.ax[1].cw[(ey * 2 + s) * 2 + 1];
          ph[2][0][s] = a.ax[2].cw[(ez * 2 + s) * 2 + 0];
          ph[2][1][s] = a.ax[2].cw[(ez * 2 + s) * 2 + 1];
        }
        const int base = fx + S1 * fy + S2 * fz;
        real t[8], dd[8], ks = 0, cs = 0;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const V4<real> r = sR[warp][base + (c & 1) + S1 * ((c >> 1) & 1) + S2 * (c >> 2)];
          t[c] = r.x;
          dd[c] = r.y;
          ks += r.z;
          cs += r.w;
        }
        if (flux) {
          const real kb = ks * (real)0.125;
          // corner differences along each axis, indexed by the other two corner bits
          real dX[2][2], dY[2][2], dZ[2][2];
#pragma unroll
          for (int b1 = 0; b1 < 2; ++b1)
#pragma unroll
            for (int b2 = 0; b2 < 2; ++b2) {
              dX[b1][b2] = t[1 + 2 * b1 + 4 * b2] - t[2 * b1 + 4 * b2];  // (ay, az)
              dY[b1][b2] = t[b1 + 2 + 4 * b2] - t[b1 + 4 * b2];          // (ax, az)
              dZ[b1][b2] = t[b1 + 2 * b2 + 4] - t[b1 + 2 * b2];          // (ax, ay)
            }
          // gradients at the Gauss points (G_x depends on (qy, qz) only, etc.)
          real Gx[2][2], Gy[2][2], Gz[2][2];
          psi2(dX, Gx);
          psi2(dY, Gy);
          psi2(dZ, Gz);
          // contraction with the coarse gradients (the factor 2 of the Gauss
          // side along the term's own axis is in cf)
          real X[2][2], Y[2][2], Z[2][2];
          contract2(ph[1], ph[2], Gx, X);
          contract2(ph[0], ph[2], Gy, Y);
          contract2(ph[0], ph[1], Gz, Z);
          const real sx = kb * a.cf[0], sy = kb * a.cf[1], sz = kb * a.cf[2];
#pragma unroll
          for (int A1 = 0; A1 < 2; ++A1)
#pragma unroll
            for (int A2 = 0; A2 < 2; ++A2) {
              const real fX = sx * X[A1][A2], fY = sy * Y[A1][A2], fZ = sz * Z[A1][A2];
              // X -> nodes (Ax, A1=Ay, A2=Az); Y -> (A1=Ax, Ay, A2=Az); Z -> (A1=Ax, A2=Ay, Az)
              acc[1 + 2 * A1 + 4 * A2] += fX;
              acc[0 + 2 * A1 + 4 * A2] -= fX;
              acc[A1 + 2 + 4 * A2] += fY;
              acc[A1 + 0 + 4 * A2] -= fY;
              acc[A1 + 2 * A2 + 4] += fZ;
              acc[A1 + 2 * A2 + 0] -= fZ;
            }
        }
        if (mass) {
          const real cb = cs * (real)0.125;
          // trilinear values at the 8 Gauss points: one 1-D psi transform per axis
          real m[8];
#pragma unroll
          for (int j = 0; j < 4; ++j) {  // x: pairs (c, c+1)
            const real d0 = dd[2 * j], d1 = dd[2 * j + 1];
            m[2 * j] = PQ * d0 + MQ * d1;
            m[2 * j + 1] = MQ * d0 + PQ * d1;
          }
#pragma unroll
          for (int j = 0; j < 4; ++j) {  // y: pairs (c, c+2)
            const int c0 = (j & 1) + 4 * (j >> 1);
            const real d0 = m[c0], d1 = m[c0 + 2];
            m[c0] = PQ * d0 + MQ * d1;
            m[c0 + 2] = MQ * d0 + PQ * d1;
          }
#pragma unroll
          for (int j = 0; j < 4; ++j) {  // z: pairs (c, c+4)
            const real d0 = m[j], d1 = m[j + 4];
            m[j] = cb * (PQ * d0 + MQ * d1);
            m[j + 4] = cb * (MQ * d0 + PQ * d1);
          }
          // contraction with the coarse shape functions, one axis at a time
#pragma unroll
          for (int j = 0; j < 4; ++j) {  // x
            const real q0 = m[2 * j], q1 = m[2 * j + 1];
            m[2 * j] = ph[0][0][0] * q0 + ph[0][0][1] * q1;
            m[2 * j + 1] = ph[0][1][0] * q0 + ph[0][1][1] * q1;
          }
#pragma unroll
          for (int j = 0; j < 4; ++j) {  // y
            const int c0 = (j & 1) + 4 * (j >> 1);
            const real q0 = m[c0], q1 = m[c0 + 2];
            m[c0] = ph[1][0][0] * q0 + ph[1][0][1] * q1;
            m[c0 + 2] = ph[1][1][0] * q0 + ph[1][1][1] * q1;
          }
#pragma unroll
          for (int j = 0; j < 4; ++j) {  // z
            const real q0 = m[j], q1 = m[j + 4];
            acc[j] -= wdt * (ph[2][0][0] * q0 + ph[2][0][1] * q1);
            acc[j + 4] -= wdt * (ph[2][1][0] * q0 + ph[2][1][1] * q1);
          }
        }
      }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) acc[i] = warp_sum(acc[i]);
    if (lane == 0) {
#pragma unroll
      for (int i = 0; i < 8; ++i) a.partials[item * 8 + i] = acc[i];
    }
    __syncwarp();
  }
}

// Sum the partials onto the coarse nodes of the box and add them into an
// output array covering the node box [ob0, ob0+on) per axis.  One thread per
// coarse node when every coarse element has one partial set; one warp per
// coarse node when the partial sets of a coarse element are many.
template <typename real>
__global__ void couple_gather_kernel(int ncbx, int ncby, int ncbz, int nchunk, int lo0, int lo1, int lo2,
                                     const real* partials, real* out, int ob0, int ob1, int ob2, int on0, int on1,
                                     real scale, const real* base) {
  pdl_begin();
  const long long tot = (long long)(ncbx + 1) * (ncby + 1) * (ncbz + 1);
  const bool per_warp = nchunk > 1;
  const int lane = threadIdx.x & 31;
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long first = per_warp ? t0 >> 5 : t0;
  const long long stride = per_warp ? ((long long)gridDim.x * blockDim.x) >> 5 : (long long)gridDim.x * blockDim.x;
  for (long long t = first; t < tot; t += stride) {
    const int bx = (int)(t % (ncbx + 1)), by = (int)((t / (ncbx + 1)) % (ncby + 1)),
              bz = (int)(t / ((long long)(ncbx + 1) * (ncby + 1)));
    real s = 0;
    const int j0 = per_warp ? lane : 0, js = per_warp ? 32 : 1;
    for (int j = j0; j < 8 * nchunk; j += js) {
      const int A = j / nchunk, c = j - A * nchunk;  // local node A of the neighbouring coarse element
      const int cx = bx - (A & 1), cy = by - ((A >> 1) & 1), cz = bz - (A >> 2);
      if (cx < 0 || cx >= ncbx || cy < 0 || cy >= ncby || cz < 0 || cz >= ncbz) continue;
      const long long base = (((long long)cz * ncby + cy) * ncbx + cx) * nchunk;
      s += partials[(base + c) * 8 + A];
    }
    if (per_warp) s = warp_sum(s);
    if (!per_warp || lane == 0) {
      const int gx = lo0 + bx - ob0, gy = lo1 + by - ob1, gz = lo2 + bz - ob2;
      const long long o = gx + (long long)gy * on0 + (long long)gz * on0 * on1;
      out[o] = (base ? base[o] : out[o]) + scale * s;
    }
  }
}

// Per-position 1-D source factors on the coarse node box:
// S[p][t] = sum_{fine e, side s assigned to coarse node t} phi_A(e,s) exp(-3 (x_q - v_p)^2 / r^2)
// One warp per table entry (row p, axis entry r): the lanes take the terms
// (coarse element r-1 or r, fine element, Gauss side) of the entry and the
// warp adds them in a fixed order.  The x entries carry the row's power
// factor cpre * P, so the assembly multiplies three table values.
template <typename real>
__global__ void coarse_source_tables(int np, const double* rows, int n0, int n1, int n2, const double* xq0,
                                     const double* xq1, const double* xq2, const real* cw0, const real* cw1,
                                     const real* cw2, const int* flo0, const int* flo1, const int* flo2,
                                     const int* fhi0, const int* fhi1, const int* fhi2, double rsq, double dsq,
                                     double cpre, real* S) {
  pdl_begin();
  const int per = (n0 + 1) + (n1 + 1) + (n2 + 1);
  const int lane = threadIdx.x & 31;
  const long long tot = (long long)np * per;
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long t = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); t < tot; t += nw) {
    const int p = (int)(t / per);
    int r = (int)(t - (long long)p * per);
    int d, ncb;
    const double* xq;
    const real* cw;
    const int *flo, *fhi;
    double s2;
    if (r < n0 + 1) {
      d = 0; ncb = n0; xq = xq0; cw = cw0; flo = flo0; fhi = fhi0; s2 = rsq;
    } else if (r < n0 + 1 + n1 + 1) {
      r -= n0 + 1; d = 1; ncb = n1; xq = xq1; cw = cw1; flo = flo1; fhi = fhi1; s2 = rsq;
    } else {
      r -= n0 + 1 + n1 + 1; d = 2; ncb = n2; xq = xq2; cw = cw2; flo = flo2; fhi = fhi2; s2 = dsq;
    }
    const double v = rows[p * 7 + d];
    const real inv2 = (real)(1.0 / s2);
    // terms of coarse element r-1 (A = 1) then r (A = 0), two Gauss sides each
    const int na = (r >= 1 && r - 1 < ncb) ? 2 * (fhi[r - 1] - flo[r - 1]) : 0;
    const int nb = (r < ncb) ? 2 * (fhi[r] - flo[r]) : 0;
    real acc = 0;
    for (int k = lane; k < na + nb; k += 32) {
      const int A = k < na ? 1 : 0;
      const int kk = k < na ? k : k - na;
      const int e = (A ? flo[r - 1] : flo[r]) + (kk >> 1), sd = kk & 1;
      const real dx = (real)(xq[e * 2 + sd] - v);  // offset in double, the rest in the kernel's precision
      acc += cw[(e * 2 + sd) * 2 + A] * exp((real)-3 * dx * dx * inv2);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) S[t] = d == 0 ? (real)(cpre * rows[p * 7 + 6]) * acc : acc;
  }
}

// Coarse node (bx, by, bz) of group g: mean over the group's np rows of
// Sx[bx] Sy[by] Sz[bz].  AG lanes per output split the rows and add their
// partial sums by a fixed shuffle tree (deterministic).
template <typename real, int AG>
__global__ void coarse_source_assemble(int np, int ng, long long gstride, int n0, int n1, int n2, int lo0, int lo1,
                                       int lo2, const real* S, real* out, int ob0, int ob1, int ob2, int on0,
                                       int on1) {
  pdl_begin();
  const int per = (n0 + 1) + (n1 + 1) + (n2 + 1);
  const int nodes = (n0 + 1) * (n1 + 1) * (n2 + 1);
  const int sub = threadIdx.x % AG;
  const long long total = (long long)nodes * ng;
  const long long tot_up = (total + 31) / 32 * 32;
  const long long stride = (long long)gridDim.x * (blockDim.x / AG);
  for (long long t = blockIdx.x * (long long)(blockDim.x / AG) + threadIdx.x / AG; t < tot_up; t += stride) {
    const bool live = t < total;
    const int g = live ? (int)(t / nodes) : 0;
    const int u = live ? (int)(t - (long long)g * nodes) : 0;
    const int bx = u % (n0 + 1), by = (u / (n0 + 1)) % (n1 + 1), bz = u / ((n0 + 1) * (n1 + 1));
    real s = 0;
    if (live)
      for (int p = g * np + sub; p < (g + 1) * np; p += AG) {
        const real* Sp = S + (long long)p * per;
        s += Sp[bx] * Sp[n0 + 1 + by] * Sp[n0 + 1 + n1 + 1 + bz];
      }
#pragma unroll
    for (int o = AG / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (live && sub == 0) {
      const int gx = lo0 + bx - ob0, gy = lo1 + by - ob1, gz = lo2 + bz - ob2;
      out[g * gstride + gx + (long long)gy * on0 + (long long)gz * on0 * on1] += s / (real)np;
    }
  }
}

inline int grid1(long long n, int block = 256) {
  long long g = (n + block - 1) / block;
  if (g > 152 * 32) g = 152 * 32;
  return g < 1 ? 1 : (int)g;
}

template <typename real>
static void fill_axes(const gm_couple_geom* g, CoupleAxis<real> ax[3], int* nchunk) {
  *nchunk = 1;
  for (int d = 0; d < 3; ++d) {
    ax[d].nfe = g->ax[d].nfe;
    ax[d].cw = (const real*)g->ax[d].cw;
    ax[d].node0 = g->ax[d].node0;
    ax[d].cb_lo = g->ax[d].cb_lo;
    ax[d].ncb = g->ax[d].ncb;
    ax[d].flo = g->ax[d].flo;
    ax[d].fhi = g->ax[d].fhi;
    ax[d].nch = cdiv(g->ax[d].rmax, SB);
    if (ax[d].nch < 1) ax[d].nch = 1;
    ax[d].invH = (real)(1.0 / g->ax[d].H);
    *nchunk *= ax[d].nch;
  }
}

// ---------------------------------------------------------------------------
// Separable coupling for constant k and rho*c.  The element sums above are
// then tensor products of 1-D maps from fine nodes to coarse nodes of the box:
//   V = k [cf0 (Dx Iy Iz) + cf1 (Ix Dy Iz) + cf2 (Ix Iy Dz)] T'
//       - (wq/dt) rho c (Ix Iy Iz)(dTa - dTb)
// with, per axis, D[N, i] = sum over fine elements e of the coarse element
// N-A (A in {0,1}) of sgn(A) (delta(i = e+1) - delta(i = e)) (the coarse
// gradient sign times the fine difference; the factor 2 of the two Gauss
// sides is in cf) and I[N, i] = sum_e sum_s cw[e,s,A] psi_s(i - e) (the
// coarse weights of the two Gauss sides times the fine linear shape
// functions).  The contraction runs one axis per kernel: fine box -> (coarse
// x, fine y, fine z) -> (coarse x, coarse y, fine z) -> coarse nodes.
// ---------------------------------------------------------------------------
template <typename real>
struct SepAxis {
  const real* cw;  // [(e*2+s)*2 + A]
  const int* flo;  // fine element range of each coarse element of the box
  const int* fhi;
  int ncb;
};

// weights of fine nodes e and e+1 in the Gauss-side sum of coarse node A
template <typename real>
__device__ __forceinline__ void side_weights(const real* cw, int e, int A, real& a0, real& a1) {
  const real PQ = (real)0.78867513459481288225, MQ = (real)0.21132486540518711775;
  const real w0 = cw[(e * 2 + 0) * 2 + A], w1 = cw[(e * 2 + 1) * 2 + A];
  a0 = w0 * PQ + w1 * MQ;
  a1 = w0 * MQ + w1 * PQ;
}

// x: U0 = Dx T', U1 = Ix T', U2 = Ix (dTa - dTb) on (coarse x, fine y, fine z).
// One warp per fine row (jy, jz): the row's T' and dTa - dTb are read once,
// coalesced, into the warp's shared-memory slice; the node weights of the
// box's fine elements (a0, a1 for A = 0, 1) are staged once per CTA; lane N
// then sums coarse node N over its fine elements.  Consecutive lanes read
// elements rmax apart; shared indices are padded (i + i/32) so that rmax = 4
// (the 5 um / 20 um ratio) reads hit 32 distinct banks.
__host__ __device__ inline int cpad(int i) { return i + (i >> 5); }

template <typename real>
__global__ void couple_sep_x(SepAxis<real> ax, SepAxis<real> ay, SepAxis<real> az, int fnx, long long fnxy,
                             const real* Tp, const real* dTa, const real* dTb, int NBy, int NBz, int nfxb, real* U,
                             long long cs) {
  pdl_begin();
  extern __shared__ __align__(16) unsigned char couple_smem[];
  const int warps = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int P = cpad(nfxb) + 1;  // padded length of one per-node or per-element array
  real* sW = reinterpret_cast<real*>(couple_smem);  // [4][P]: a0(A=0), a1(A=0), a0(A=1), a1(A=1)
  real* sF = sW + 4 * P + (long long)warp * 2 * P;   // [2][P]: T', dTa - dTb of the row
  const int ncx = ax.ncb;
  const int fx0 = ax.flo[0], nfx = ax.fhi[ncx - 1] - fx0 + 1;  // fine nodes of the box along x (<= nfxb)
  const int fy0 = ay.flo[0], fz0 = az.flo[0];
  const int nfy = ay.fhi[ay.ncb - 1] - fy0 + 1, nfz = az.fhi[az.ncb - 1] - fz0 + 1;
  for (int le = threadIdx.x; le < nfx - 1; le += blockDim.x) {
#pragma unroll
    for (int A = 0; A < 2; ++A) {
      real a0, a1;
      side_weights(ax.cw, fx0 + le, A, a0, a1);
      sW[(2 * A) * P + cpad(le)] = a0;
      sW[(2 * A + 1) * P + cpad(le)] = a1;
    }
  }
  __syncthreads();
  const long long nrows = (long long)NBy * NBz;
  for (long long row = (long long)blockIdx.x * warps + warp; row < nrows; row += (long long)gridDim.x * warps) {
    const int jy = (int)(row % NBy), jz = (int)(row / NBy);
    if (jy >= nfy || jz >= nfz) continue;  // the same for the whole warp
    const long long base = fx0 + (long long)(fy0 + jy) * fnx + (fz0 + jz) * fnxy;
    for (int i = lane; i < nfx; i += 32) {
      sF[cpad(i)] = Tp ? Tp[base + i] : (real)0;
      sF[P + cpad(i)] = dTa ? dTa[base + i] - dTb[base + i] : (real)0;
    }
    __syncwarp();
    for (int Nx = lane; Nx <= ncx; Nx += 32) {
      real uD = 0, uI = 0, uM = 0;
#pragma unroll
      for (int A = 1; A >= 0; --A) {
        const int c = Nx - A;
        if (c < 0 || c >= ncx) continue;
        const real sg = A ? (real)1 : (real)-1;
        const real* w0 = sW + (2 * A) * P;
        const real* w1 = sW + (2 * A + 1) * P;
        const int e1 = ax.fhi[c] - fx0;
        for (int le = ax.flo[c] - fx0; le < e1; ++le) {
          const int q0 = cpad(le), q1 = cpad(le + 1);
          const real a0 = w0[q0], a1 = w1[q0];
          const real t0 = sF[q0], t1 = sF[q1];
          uD += sg * (t1 - t0);
          uI += a0 * t0 + a1 * t1;
          uM += a0 * sF[P + q0] + a1 * sF[P + q1];
        }
      }
      const long long t = row * (ncx + 1) + Nx;
      U[t] = uD;
      U[cs + t] = uI;
      U[2 * cs + t] = uM;
    }
    __syncwarp();
  }
}

// The y and z contractions give each output CSUB lanes: lane j of the group
// takes the j-th, (j+CSUB)-th, ... fine element of the node's list (the
// elements of coarse element N-1 with A = 1, then those of N with A = 0), and
// the group's partial sums are added by a fixed shuffle tree (deterministic).
constexpr int CSUB = 4;

template <typename real>
__device__ __forceinline__ real csub_sum(real v) {
#pragma unroll
  for (int o = CSUB / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// element k of coarse node N's list: sets (e, A); false past the end
template <typename real>
__device__ __forceinline__ bool node_elem(const SepAxis<real>& ax, int N, int k, int& e, int& A) {
  if (N >= 1) {
    const int n1 = ax.fhi[N - 1] - ax.flo[N - 1];
    if (k < n1) {
      e = ax.flo[N - 1] + k;
      A = 1;
      return true;
    }
    k -= n1;
  }
  if (N < ax.ncb && k < ax.fhi[N] - ax.flo[N]) {
    e = ax.flo[N] + k;
    A = 0;
    return true;
  }
  return false;
}

// y: W0 = Iy U0, W1 = Dy U1, W2 = Iy U1, W3 = Iy U2 on (coarse x, coarse y, fine z)
template <typename real>
__global__ void couple_sep_y(int ncx, SepAxis<real> ay, SepAxis<real> az, int NBy, int NBz, const real* U,
                             long long cs, bool flux, bool mass, real* W, long long ws) {
  pdl_begin();
  const int ncy = ay.ncb;
  const long long n = (long long)(ncx + 1) * (ncy + 1) * NBz;
  const int fy0 = ay.flo[0], fz0 = az.flo[0];
  const int nfz = az.fhi[az.ncb - 1] - fz0 + 1;
  const int sub = threadIdx.x % CSUB;
  // the loop runs the same number of times in every lane group of a warp
  const long long stride = (long long)gridDim.x * (blockDim.x / CSUB);
  const long long t_first = blockIdx.x * (long long)(blockDim.x / CSUB) + threadIdx.x / CSUB;
  const long long n_up = (n + 31) / 32 * 32;
  for (long long t = t_first; t < n_up; t += stride) {
    real w0 = 0, w1 = 0, w2 = 0, w3 = 0;
    const bool live = t < n;
    const int Nx = (int)(t % (ncx + 1));
    const long long r = t / (ncx + 1);
    const int Ny = (int)(r % (ncy + 1)), jz = (int)(r / (ncy + 1));
    if (live && jz < nfz) {
      int e, A;
      for (int k = sub; node_elem(ay, Ny, k, e, A); k += CSUB) {
        real a0, a1;
        side_weights(ay.cw, e, A, a0, a1);
        const real sg = A ? (real)1 : (real)-1;
        const long long i0 = ((long long)jz * NBy + (e - fy0)) * (ncx + 1) + Nx, i1 = i0 + (ncx + 1);
        if (flux) {
          const real d0 = U[i0], d1 = U[i1], u0 = U[cs + i0], u1 = U[cs + i1];
          w0 += a0 * d0 + a1 * d1;
          w1 += sg * (u1 - u0);
          w2 += a0 * u0 + a1 * u1;
        }
        if (mass) w3 += a0 * U[2 * cs + i0] + a1 * U[2 * cs + i1];
      }
    }
    w0 = csub_sum(w0);
    w1 = csub_sum(w1);
    w2 = csub_sum(w2);
    w3 = csub_sum(w3);
    if (live && sub == 0) {
      W[t] = w0;
      W[ws + t] = w1;
      W[2 * ws + t] = w2;
      W[3 * ws + t] = w3;
    }
  }
}

// z: the coarse nodes; out[box node] += scale * V
template <typename real>
__global__ void couple_sep_z(int ncx, int ncy, SepAxis<real> az, int lo0, int lo1, int lo2, const real* W,
                             long long ws, bool flux, bool mass, real kcf0, real kcf1, real kcf2, const double* dt,
                             real mwq, real* out, int ob0, int ob1, int ob2, int on0, int on1, real scale,
                             const real* base) {
  pdl_begin();
  const int ncz = az.ncb;
  const long long n = (long long)(ncx + 1) * (ncy + 1) * (ncz + 1);
  const int fz0 = az.flo[0];
  const real mf = mass ? mwq / (real)(*dt) : (real)0;  // (wq/dt) rho c
  const long long pl = (long long)(ncx + 1) * (ncy + 1);
  const int sub = threadIdx.x % CSUB;
  const long long stride = (long long)gridDim.x * (blockDim.x / CSUB);
  const long long t_first = blockIdx.x * (long long)(blockDim.x / CSUB) + threadIdx.x / CSUB;
  const long long n_up = (n + 31) / 32 * 32;
  for (long long t = t_first; t < n_up; t += stride) {
    real v = 0;
    const bool live = t < n;
    const int Nx = (int)(t % (ncx + 1)), Ny = (int)((t / (ncx + 1)) % (ncy + 1)), Nz = (int)(t / pl);
    if (live) {
      int e, A;
      for (int k = sub; node_elem(az, Nz, k, e, A); k += CSUB) {
        real a0, a1;
        side_weights(az.cw, e, A, a0, a1);
        const real sg = A ? (real)1 : (real)-1;
        const long long i0 = (long long)(e - fz0) * pl + (long long)Ny * (ncx + 1) + Nx, i1 = i0 + pl;
        if (flux)
          v += kcf0 * (a0 * W[i0] + a1 * W[i1]) + kcf1 * (a0 * W[ws + i0] + a1 * W[ws + i1]) +
               kcf2 * sg * (W[2 * ws + i1] - W[2 * ws + i0]);
        if (mass) v -= mf * (a0 * W[3 * ws + i0] + a1 * W[3 * ws + i1]);
      }
    }
    v = csub_sum(v);
    if (live && sub == 0) {
      const int gx = lo0 + Nx - ob0, gy = lo1 + Ny - ob1, gz = lo2 + Nz - ob2;
      const long long o = gx + (long long)gy * on0 + (long long)gz * on0 * on1;
      out[o] = (base ? base[o] : out[o]) + scale * v;
    }
  }
}

// Scratch of the separable path: U (3 channels over coarse x, fine y, fine z)
// and W (4 channels over coarse x, coarse y, fine z), fine extents bounded by
// ncb * rmax + 1 per axis.
// x-kernel CTA shape: warps a CTA and dynamic shared memory (bytes), 0 warps
// when one fine row does not fit.
static void sep_x_shape(const gm_couple_geom* g, size_t esz, int* warps, size_t* smem) {
  const long long nfxb = (long long)g->ax[0].ncb * g->ax[0].rmax + 1;
  const long long P = cpad((int)nfxb) + 1;
  const long long fixed = 4 * P * (long long)esz, per = 2 * P * (long long)esz;
  *warps = 0;
  for (int w = 8; w >= 1; w >>= 1)
    if (fixed + w * per <= 48 * 1024) {
      *warps = w;
      break;
    }
  *smem = (size_t)(fixed + *warps * per);
}

static void sep_extents(const gm_couple_geom* g, long long* cs, long long* ws, int* NBy, int* NBz) {
  *NBy = g->ax[1].ncb * g->ax[1].rmax + 1;
  *NBz = g->ax[2].ncb * g->ax[2].rmax + 1;
  *cs = (long long)(g->ax[0].ncb + 1) * *NBy * *NBz;
  *ws = (long long)(g->ax[0].ncb + 1) * (g->ax[1].ncb + 1) * *NBz;
}

static long long sep_scratch(const gm_couple_geom* g) {
  long long cs, ws;
  int NBy, NBz;
  sep_extents(g, &cs, &ws, &NBy, &NBz);
  return 3 * cs + 4 * ws;
}

static bool geom_ok(const gm_couple_geom* g) {
  for (int d = 0; d < 3; ++d) {
    const gm_couple_axis& a = g->ax[d];
    if (a.nfe < 1 || a.ncb < 1 || !a.cw || !a.flo || !a.fhi || a.rmax < 1 || !(a.H > 0)) return false;
  }
  return true;
}

}  // namespace gm

using namespace gm;

static long long element_scratch(const gm_couple_geom* g) {
  long long items = 1;
  for (int d = 0; d < 3; ++d) items *= (long long)g->ax[d].ncb * cdiv(g->ax[d].rmax, SB);
  return items * 8;
}

extern "C" long long gm_couple_partials_size(const gm_couple_geom* g) {
  if (!g || !geom_ok(g)) return -1;
  const long long a = element_scratch(g), b = sep_scratch(g);
  return a > b ? a : b;
}

template <typename real>
static int do_couple_sep(const gm_couple_args* g, const gm_props* pr, cudaStream_t st) {
  SepAxis<real> ax[3];
  for (int d = 0; d < 3; ++d) {
    ax[d].cw = (const real*)g->geom.ax[d].cw;
    ax[d].flo = g->geom.ax[d].flo;
    ax[d].fhi = g->geom.ax[d].fhi;
    ax[d].ncb = g->geom.ax[d].ncb;
  }
  long long cs, ws;
  int NBy, NBz;
  sep_extents(&g->geom, &cs, &ws, &NBy, &NBz);
  real* U = (real*)g->partials;
  real* W = U + 3 * cs;
  const bool flux = g->Tp != nullptr, mass = g->dTa != nullptr;
  const long long fnxy = (long long)g->fine_nodes[0] * g->fine_nodes[1];
  int xw;
  size_t xsm;
  sep_x_shape(&g->geom, sizeof(real), &xw, &xsm);
  if (xw < 1) return GM_ERR_TOO_LARGE;
  const int nfxb = g->geom.ax[0].ncb * g->geom.ax[0].rmax + 1;
  const long long rows = (long long)NBy * NBz;
  if (launch_k(couple_sep_x<real>, dim3(grid1(rows, xw)), dim3(32 * xw), xsm, st, ax[0], ax[1], ax[2],
               g->fine_nodes[0], fnxy, (const real*)g->Tp, (const real*)g->dTa, (const real*)g->dTb, NBy, NBz, nfxb,
               U, cs) != cudaSuccess)
    return GM_ERR_LAUNCH;
  if (launch_k(couple_sep_y<real>, dim3(grid1(ws * CSUB)), dim3(256), 0, st, ax[0].ncb, ax[1], ax[2], NBy, NBz,
               (const real*)U, cs, flux, mass, W, ws) != cudaSuccess)
    return GM_ERR_LAUNCH;
  const double wq = g->fine_h[0] * g->fine_h[1] * g->fine_h[2] / 8.0;
  const double kc = pr->k_fluid / 1000.0;
  double kcf[3];
  for (int d = 0; d < 3; ++d) kcf[d] = kc * (-2.0 * wq / (g->geom.ax[d].H * g->fine_h[d]));
  const long long nodes = (long long)(ax[0].ncb + 1) * (ax[1].ncb + 1) * (ax[2].ncb + 1);
  if (launch_k(couple_sep_z<real>, dim3(grid1(nodes * CSUB)), dim3(256), 0, st, ax[0].ncb, ax[1].ncb, ax[2],
               g->geom.ax[0].cb_lo, g->geom.ax[1].cb_lo, g->geom.ax[2].cb_lo, (const real*)W, ws, flux, mass,
               (real)kcf[0], (real)kcf[1], (real)kcf[2], g->dt, (real)(wq * pr->rho * pr->cp_fluid),
               (real*)g->out, g->out_lo[0], g->out_lo[1], g->out_lo[2], g->out_n[0], g->out_n[1],
               (real)g->scale, (const real*)g->base) != cudaSuccess)
    return GM_ERR_LAUNCH;
  return GM_OK;
}

template <typename real>
static int do_couple(const gm_couple_args* g, const gm_props* pr, cudaStream_t st) {
  CoupleK<real> a;
  fill_axes<real>(&g->geom, a.ax, &a.nchunk);
  a.fnx = g->fine_nodes[0];
  a.fny = g->fine_nodes[1];
  a.T = (const real*)g->T;
  a.ph = g->ph;
  a.substrate = g->substrate;
  a.k_arr = (const real*)g->k_arr;
  a.rc_arr = (const real*)g->rc_arr;
  a.Tp = (const real*)g->Tp;
  a.dTa = (const real*)g->dTa;
  a.dTb = (const real*)g->dTb;
  a.dt = g->dt;
  a.wq = (real)(g->fine_h[0] * g->fine_h[1] * g->fine_h[2] / 8.0);
  for (int d = 0; d < 3; ++d)
    a.cf[d] = (real)(-2.0 * (g->fine_h[0] * g->fine_h[1] * g->fine_h[2] / 8.0) / (g->geom.ax[d].H * g->fine_h[d]));
  a.partials = (real*)g->partials;
  a.nitems = (long long)a.ax[0].ncb * a.ax[1].ncb * a.ax[2].ncb * a.nchunk;
  a.p = make_props<real>(*pr);
  a.kconst = !g->k_arr && pr->k_powder == pr->k_bulk_a0 && pr->k_fluid == pr->k_bulk_a0 && pr->k_bulk_a1 == 0.0 &&
             pr->cp_solid_a1 == 0.0 && pr->cp_mushy == pr->cp_solid_a0 && pr->cp_fluid == pr->cp_solid_a0;
  long long blocks = (a.nitems + 3) / 4;
  if (blocks > 152 * 16) blocks = 152 * 16;
  launch_k(couple_kernel<real>, dim3((int)blocks), dim3(128), 0, st, a);
  if (cudaGetLastError() != cudaSuccess) return GM_ERR_LAUNCH;
  const int ncbx = a.ax[0].ncb, ncby = a.ax[1].ncb, ncbz = a.ax[2].ncb;
  const long long nodes = (long long)(ncbx + 1) * (ncby + 1) * (ncbz + 1);
  launch_k(couple_gather_kernel<real>, dim3(grid1(a.nchunk > 1 ? nodes * 32 : nodes)), dim3(256), 0, st,
      ncbx, ncby, ncbz, a.nchunk, g->geom.ax[0].cb_lo, g->geom.ax[1].cb_lo, g->geom.ax[2].cb_lo, a.partials,
      (real*)g->out, g->out_lo[0], g->out_lo[1], g->out_lo[2], g->out_n[0], g->out_n[1], (real)g->scale,
      (const real*)g->base);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

static bool box_inside(const gm_couple_geom* g, const int lo[3], const int n[3]) {
  for (int d = 0; d < 3; ++d) {
    if (g->ax[d].cb_lo < lo[d] || g->ax[d].cb_lo + g->ax[d].ncb + 1 > lo[d] + n[d]) return false;
  }
  return true;
}

extern "C" int gm_couple(const gm_couple_args* g, const gm_props* p, void* stream) {
  if (!g || !p || !geom_ok(&g->geom) || !g->T || !g->out || !g->partials) return GM_ERR_ARG;
  if (!g->Tp && !g->dTa) return GM_ERR_ARG;
  if ((g->dTa == nullptr) != (g->dTb == nullptr) || (g->dTa && !g->dt)) return GM_ERR_ARG;
  if ((g->k_arr == nullptr) != (g->rc_arr == nullptr)) return GM_ERR_ARG;
  if (!box_inside(&g->geom, g->out_lo, g->out_n)) return GM_ERR_ARG;
  if (g->base) {  // out = base + terms: every node of the output box must be a coupling node
    for (int d = 0; d < 3; ++d)
      if (g->out_lo[d] != g->geom.ax[d].cb_lo || g->out_n[d] != g->geom.ax[d].ncb + 1) return GM_ERR_ARG;
    if (g->base == g->out) return GM_ERR_ARG;
  }
  if ((long long)g->fine_nodes[0] * g->fine_nodes[1] * g->fine_nodes[2] >= (1LL << 31)) return GM_ERR_TOO_LARGE;
  if (g->method < 0 || g->method > 2) return GM_ERR_ARG;
  const bool kconst = !g->k_arr && p->k_powder == p->k_bulk_a0 && p->k_fluid == p->k_bulk_a0 &&
                      p->k_bulk_a1 == 0.0 && p->cp_solid_a1 == 0.0 && p->cp_mushy == p->cp_solid_a0 &&
                      p->cp_fluid == p->cp_solid_a0;
  if (g->method == 2 && !kconst) return GM_ERR_ARG;
  int xw;
  size_t xsm;
  sep_x_shape(&g->geom, g->dtype == GM_F64 ? 8 : 4, &xw, &xsm);
  if (g->method == 2 && xw < 1) return GM_ERR_TOO_LARGE;
  const bool sep =
      g->method == 2 || (g->method == 0 && kconst && xw >= 1 && sep_scratch(&g->geom) <= g->partials_cap);
  const long long need = sep ? sep_scratch(&g->geom) : element_scratch(&g->geom);
  if (need > g->partials_cap) return GM_ERR_TOO_LARGE;
  cudaStream_t st = (cudaStream_t)stream;
  if (sep) return g->dtype == GM_F32 ? do_couple_sep<float>(g, p, st) : do_couple_sep<double>(g, p, st);
  if (g->dtype == GM_F32) return do_couple<float>(g, p, st);
  if (g->dtype == GM_F64) return do_couple<double>(g, p, st);
  return GM_ERR_ARG;
}

template <typename real>
static int do_source(const gm_coarse_source_args* g, const gm_props* pr, cudaStream_t st) {
  const gm_couple_geom& G = g->geom;
  const int n0 = G.ax[0].ncb, n1 = G.ax[1].ncb, n2 = G.ax[2].ncb;
  const long long tabs = (long long)g->npos * ((n0 + 1) + (n1 + 1) + (n2 + 1));
  const double r = pr->laser_radius, d = pr->laser_depth;
  const double rc = 1.0 / (r * sqrt(M_PI)), dc = 1.0 / (d * sqrt(M_PI));
  const double cpre = 6.0 * sqrt(3.0) * pr->laser_eta * rc * rc * dc * g->fine_wq;
  launch_k(coarse_source_tables<real>, dim3(grid1(tabs * 32)), dim3(256), 0, st,
      g->npos, g->rows, n0, n1, n2, g->xq[0], g->xq[1], g->xq[2], (const real*)G.ax[0].cw,
      (const real*)G.ax[1].cw, (const real*)G.ax[2].cw, G.ax[0].flo, G.ax[1].flo, G.ax[2].flo, G.ax[0].fhi,
      G.ax[1].fhi, G.ax[2].fhi, r * r, d * d, cpre, (real*)g->scratch);
  if (cudaGetLastError() != cudaSuccess) return GM_ERR_LAUNCH;
  const long long nodes = (long long)(n0 + 1) * (n1 + 1) * (n2 + 1);
  const int ng = g->ngroups > 1 ? g->ngroups : 1;
  const int np = g->npos / ng;
  if (np >= 16)
    launch_k(coarse_source_assemble<real, 32>, dim3(grid1(nodes * ng * 32)), dim3(256), 0, st, np, ng,
             g->out_group_stride, n0, n1, n2, G.ax[0].cb_lo, G.ax[1].cb_lo, G.ax[2].cb_lo, (const real*)g->scratch,
             (real*)g->out, g->out_lo[0], g->out_lo[1], g->out_lo[2], g->out_n[0], g->out_n[1]);
  else
    launch_k(coarse_source_assemble<real, 4>, dim3(grid1(nodes * ng * 4)), dim3(256), 0, st, np, ng,
             g->out_group_stride, n0, n1, n2, G.ax[0].cb_lo, G.ax[1].cb_lo, G.ax[2].cb_lo, (const real*)g->scratch,
             (real*)g->out, g->out_lo[0], g->out_lo[1], g->out_lo[2], g->out_n[0], g->out_n[1]);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_coarse_source(const gm_coarse_source_args* g, const gm_props* p, void* stream) {
  if (!g || !p || !geom_ok(&g->geom) || !g->rows || g->npos < 1 || !g->out || !g->scratch) return GM_ERR_ARG;
  if (!g->xq[0] || !g->xq[1] || !g->xq[2]) return GM_ERR_ARG;
  if (!box_inside(&g->geom, g->out_lo, g->out_n)) return GM_ERR_ARG;
  if (g->ngroups > 1 && (g->npos % g->ngroups ||
                         g->out_group_stride < (long long)g->out_n[0] * g->out_n[1] * g->out_n[2]))
    return GM_ERR_ARG;
  const gm_couple_geom& G = g->geom;
  const long long need = (long long)g->npos * ((G.ax[0].ncb + 1) + (G.ax[1].ncb + 1) + (G.ax[2].ncb + 1));
  if (need > g->scratch_cap) return GM_ERR_TOO_LARGE;
  cudaStream_t st = (cudaStream_t)stream;
  if (g->dtype == GM_F32) return do_source<float>(g, p, st);
  if (g->dtype == GM_F64) return do_source<double>(g, p, st);
  return GM_ERR_ARG;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of gm_couple.
//
// Some callers cannot allocate device memory at the moment they need the
// coupling terms: code that runs while a framework owns the device allocator
// (for example inside another runtime's custom call), a loop that must not
// pay the device-wide synchronisation that cudaMalloc/cudaFree can imply, or
// code that has no way to keep a scratch buffer alive between calls.  For
// them gm_couple_noalloc keeps gm_couple's partial sums in this fixed array,
// which every GPU that loads the library holds until the process exits.
// ---------------------------------------------------------------------------
#include <mutex>

static __device__ __align__(256) unsigned char g_couple_scratch[GM_COUPLE_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

// Device address of g_couple_scratch on the current device, looked up once per
// device (host code cannot use the symbol itself as a device pointer).  The
// look-up is refused while `stream` is being captured: a first call inside a
// capture would otherwise run cudaGetSymbolAddress in the middle of it.
int scratch_address(void* stream, void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GM_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (g_scratch_addr[dev] == nullptr) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing((cudaStream_t)stream, &cs) != cudaSuccess) return GM_ERR_CUDA;
    if (cs != cudaStreamCaptureStatusNone) return GM_ERR_ARG;  // first call on this device during a capture
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_couple_scratch) != cudaSuccess || p == nullptr) return GM_ERR_CUDA;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return GM_OK;
}
}  // namespace

extern "C" int gm_couple_noalloc(const gm_couple_args* g, const gm_props* p, void* stream) {
  if (!g || !p || !geom_ok(&g->geom)) return GM_ERR_ARG;
  if (g->dtype != GM_F32 && g->dtype != GM_F64) return GM_ERR_ARG;
  const size_t esz = g->dtype == GM_F64 ? sizeof(double) : sizeof(float);
  void* scratch = nullptr;
  const int rc = scratch_address(stream, &scratch);
  if (rc != GM_OK) return rc;
  // Same arguments with the library's array as the partials: gm_couple picks
  // its path against this capacity (the separable contraction when it fits,
  // else the element reduction) and returns GM_ERR_TOO_LARGE when the path it
  // takes needs more than the array holds.
  gm_couple_args a = *g;
  a.partials = scratch;
  a.partials_cap = (long long)(GM_COUPLE_NOALLOC_SCRATCH_BYTES / esz);
  return gm_couple(&a, p, stream);
}
