// Diagnostics of one level window, reduced in FP64 on the device:
//   * energy balance over an interval (the check that decides whether a
//     predicted Level-3 field is accepted),
//   * melt-pool extent at an isotherm (length / width / depth),
//   * max and RMS difference of two fields (FP32 run against an FP64 run).
// The reference has no counterpart; the quantities are defined here and in
// include/gomelt.h.  Every reduction is two-stage (per-block partials, then
// one block in a fixed order), so results are deterministic.
#include <math.h>

#include "gm_common.cuh"

namespace gm {

constexpr int DG_BLOCK = 256;
constexpr int DG_GRID = 152 * 4;  // blocks of the first stage (partials per quantity)

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double wmin(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double wmax(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block reduction of NV values with per-value operation op (0 sum, 1 min,
// 2 max); thread 0 returns the results in v.
template <int NV>
__device__ void block_reduce(double (&v)[NV], const int (&op)[NV]) {
  __shared__ double sh[NV][DG_BLOCK / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    v[j] = op[j] == 0 ? wsum(v[j]) : (op[j] == 1 ? wmin(v[j]) : wmax(v[j]));
    if (lane == 0) sh[j][w] = v[j];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double r = sh[j][0];
      for (int i = 1; i < DG_BLOCK / 32; ++i)
        r = op[j] == 0 ? r + sh[j][i] : (op[j] == 1 ? fmin(r, sh[j][i]) : fmax(r, sh[j][i]));
      v[j] = r;
    }
  }
  __syncthreads();
}

template <typename real>
__device__ __forceinline__ double ld(const void* p, long long i) {
  return (double)((const real*)p)[i];
}

// ---------------------------------------------------------------------------
// Energy balance.  Element pass: stored heat, conduction and surface flux of
// the interior nodes, with T_bar = (T0 + T1) / 2.
// ---------------------------------------------------------------------------
struct EnergyK {
  int nx, ny, nz, ne_planes, dtype;
  double hx, hy, hz;
  const void* T0;
  const void* T1;
  const uint8_t* ph;
  long long substrate;
  double lam[8], wvol, w2;
  Props<double> p;
};

// Volumetric enthalpy rho * integral of c_p from 0 to T for the phase model's
// heat capacity (computeStateProperties, :2567-2614): c_p = c1 T + c0 up to
// T_solidus, c_mushy between T_solidus and T_liquidus, c_fluid above.
__device__ __forceinline__ double enthalpy(const Props<double>& p, double T) {
  const double Ts = p.T_solidus, Tl = p.T_liquidus;
  const double Hs = p.cp_solid_a0 * Ts + 0.5 * p.cp_solid_a1 * Ts * Ts;
  double H;
  if (T <= Ts)
    H = p.cp_solid_a0 * T + 0.5 * p.cp_solid_a1 * T * T;
  else if (T < Tl)
    H = Hs + p.cp_mushy * (T - Ts);
  else
    H = Hs + p.cp_mushy * (Tl - Ts) + p.cp_fluid * (T - Tl);
  return p.rho * H;
}

__device__ __forceinline__ bool interior(int ix, int iy, int iz, int nx, int ny, int ne_planes) {
  return ix >= 1 && ix <= nx - 2 && iy >= 1 && iy <= ny - 2 && iz >= 1 && iz <= ne_planes;
}

template <typename real>
__global__ void __launch_bounds__(DG_BLOCK) energy_elem_kernel(const EnergyK a, double* part) {
  const double PQ = 0.78867513459481288225, MQ = 0.21132486540518711775;
  const int ex_n = a.nx - 1, ey_n = a.ny - 1;
  const long long ne = (long long)ex_n * ey_n * a.ne_planes;
  const long long nxy = (long long)a.nx * a.ny;
  double es = 0, ec = 0, ef = 0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ne; e += (long long)gridDim.x * blockDim.x) {
    const int ex = (int)(e % ex_n), ey = (int)((e / ex_n) % ey_n), ez = (int)(e / ((long long)ex_n * ey_n));
    double t0[8], t1[8], tb[8], R[8], ks = 0;
    bool in[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int ix = ex + (c & 1), iy = ey + ((c >> 1) & 1), iz = ez + (c >> 2);
      const long long id = ix + iy * (long long)a.nx + iz * nxy;
      t0[c] = ld<real>(a.T0, id);
      t1[c] = ld<real>(a.T1, id);
      tb[c] = 0.5 * (t0[c] + t1[c]);
      double k, rc;
      node_props_sel<double>(a.p, tb[c], a.ph ? (uint32_t)a.ph[id] : 0u, id < a.substrate, k, rc);
      ks += k;
      in[c] = interior(ix, iy, iz, a.nx, a.ny, a.ne_planes);
      R[c] = tb[c];
    }
    const double kbar = ks * 0.125;
    bfly_fwd(R);
#pragma unroll
    for (int m = 0; m < 8; ++m) R[m] *= a.lam[m] * kbar;
    bfly_inv(R);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      if (in[c]) {
        es += a.wvol * (enthalpy(a.p, t1[c]) - enthalpy(a.p, t0[c]));
        ec -= R[c];
      }
    }
    if (ez == a.ne_planes - 1) {
#pragma unroll
      for (int qy = 0; qy < 2; ++qy)
#pragma unroll
        for (int qx = 0; qx < 2; ++qx) {
          const double px0 = qx ? MQ : PQ, px1 = qx ? PQ : MQ;
          const double py0 = qy ? MQ : PQ, py1 = qy ? PQ : MQ;
          const double Tq = px0 * py0 * tb[4] + px1 * py0 * tb[5] + px0 * py1 * tb[6] + px1 * py1 * tb[7];
          const double q = surface_flux<double>(a.p, Tq) * a.w2;
          if (in[4]) ef += px0 * py0 * q;
          if (in[5]) ef += px1 * py0 * q;
          if (in[6]) ef += px0 * py1 * q;
          if (in[7]) ef += px1 * py1 * q;
        }
    }
  }
  double v[3] = {es, ec, ef};
  const int op[3] = {0, 0, 0};
  block_reduce<3>(v, op);
  if (threadIdx.x == 0) {
    part[blockIdx.x * 3 + 0] = v[0];
    part[blockIdx.x * 3 + 1] = v[1];
    part[blockIdx.x * 3 + 2] = v[2];
  }
}

// Laser energy deposited at the interior nodes: per fine step r,
// dt_r * c * P_r * (sum Sx)(sum Sy)(sum Sz) over the interior index ranges.
// One block per row.
__global__ void __launch_bounds__(DG_BLOCK) energy_source_kernel(int nx, int ny, int nz, int ne_planes, double ox,
                                                                double oy, double oz, double hx, double hy,
                                                                double hz, const double* rows, double inv_r2,
                                                                double inv_d2, double src_c, double* part) {
  const double* row = rows + blockIdx.x * 7;
  const double rx = ox - row[0], ry = oy - row[1], rz = oz - row[2];
  double v[3] = {0, 0, 0};
  for (int i = threadIdx.x; i < nx + ny + nz; i += blockDim.x) {
    if (i < nx) {
      if (i >= 1 && i <= nx - 2) v[0] += src_factor<double>(i, nx, rx, hx, inv_r2);
    } else if (i < nx + ny) {
      const int j = i - nx;
      if (j >= 1 && j <= ny - 2) v[1] += src_factor<double>(j, ny, ry, hy, inv_r2);
    } else {
      const int k = i - nx - ny;
      // active elements only: element planes [0, ne_planes)
      if (k >= 1 && k <= ne_planes) v[2] += src_factor<double>(k, ne_planes + 1, rz, hz, inv_d2);
    }
  }
  const int op[3] = {0, 0, 0};
  block_reduce<3>(v, op);
  if (threadIdx.x == 0) part[blockIdx.x] = row[5] * src_c * row[6] * v[0] * v[1] * v[2];
}

// out = {stored, source, surface, conduction}; the element partials are
// summed in block order, the source terms in row order.
__global__ void energy_final_kernel(const double* part, int nblk, const double* spart, int npos, double interval,
                                    double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double es = 0, ec = 0, ef = 0, src = 0;
  for (int b = 0; b < nblk; ++b) {
    es += part[b * 3 + 0];
    ec += part[b * 3 + 1];
    ef += part[b * 3 + 2];
  }
  for (int r = 0; r < npos; ++r) src += spart[r];
  out[0] = es;
  out[1] = src;
  out[2] = interval * ef;
  out[3] = interval * ec;
}

// ---------------------------------------------------------------------------
// Melt-pool extent: nodes with T >= iso, extended to the linearly
// interpolated isotherm crossing towards each colder neighbour.
// ---------------------------------------------------------------------------
template <typename real>
__global__ void __launch_bounds__(DG_BLOCK) meltpool_kernel(int nx, int ny, int nz, double ox, double oy, double oz,
                                                           double hx, double hy, double hz, const void* Tv, double iso,
                                                           double* part) {
  const real* T = (const real*)Tv;
  const long long nxy = (long long)nx * ny, n = nxy * nz;
  double v[7] = {INFINITY, -INFINITY, INFINITY, -INFINITY, INFINITY, -INFINITY, 0.0};
  const int op[7] = {1, 2, 1, 2, 1, 2, 0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double t = (double)T[i];
    if (!(t >= iso)) continue;
    const int ix = (int)(i % nx), iy = (int)((i / nx) % ny), iz = (int)(i / nxy);
    const int idx[3] = {ix, iy, iz}, nn[3] = {nx, ny, nz};
    const long long st[3] = {1, nx, nxy};
    const double o[3] = {ox, oy, oz}, h[3] = {hx, hy, hz};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double x = o[d] + h[d] * idx[d];
      double lo = x, hi = x;
      if (idx[d] > 0) {
        const double tn = (double)T[i - st[d]];
        if (tn < iso) lo = x - h[d] * (t - iso) / (t - tn);
      }
      if (idx[d] < nn[d] - 1) {
        const double tn = (double)T[i + st[d]];
        if (tn < iso) hi = x + h[d] * (t - iso) / (t - tn);
      }
      v[2 * d] = fmin(v[2 * d], lo);
      v[2 * d + 1] = fmax(v[2 * d + 1], hi);
    }
    v[6] += 1.0;
  }
  block_reduce<7>(v, op);
  if (threadIdx.x == 0)
    for (int j = 0; j < 7; ++j) part[blockIdx.x * 7 + j] = v[j];
}

__global__ void meltpool_final_kernel(const double* part, int nblk, double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double v[7] = {INFINITY, -INFINITY, INFINITY, -INFINITY, INFINITY, -INFINITY, 0.0};
  for (int b = 0; b < nblk; ++b) {
    for (int j = 0; j < 6; ++j) v[j] = (j & 1) ? fmax(v[j], part[b * 7 + j]) : fmin(v[j], part[b * 7 + j]);
    v[6] += part[b * 7 + 6];
  }
  for (int j = 0; j < 7; ++j) out[j] = v[j];
}

// ---------------------------------------------------------------------------
// Field difference: max |a - b| and sum (a - b)^2, then RMS.
// ---------------------------------------------------------------------------
template <typename ra, typename rb>
__global__ void __launch_bounds__(DG_BLOCK) field_err_kernel(long long n, const void* A, const void* B, double* part) {
  double v[2] = {0, 0};
  const int op[2] = {2, 0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double d = ld<ra>(A, i) - ld<rb>(B, i);
    v[0] = fmax(v[0], fabs(d));
    v[1] += d * d;
  }
  block_reduce<2>(v, op);
  if (threadIdx.x == 0) {
    part[blockIdx.x * 2] = v[0];
    part[blockIdx.x * 2 + 1] = v[1];
  }
}

__global__ void field_err_final_kernel(const double* part, int nblk, long long n, double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double m = 0, s = 0;
  for (int b = 0; b < nblk; ++b) {
    m = fmax(m, part[b * 2]);
    s += part[b * 2 + 1];
  }
  out[0] = m;
  out[1] = n > 0 ? sqrt(s / (double)n) : 0.0;
}

inline int dgrid(long long n) {
  long long g = (n + DG_BLOCK - 1) / DG_BLOCK;
  if (g > DG_GRID) g = DG_GRID;
  return g < 1 ? 1 : (int)g;
}

}  // namespace gm

using namespace gm;

extern "C" long long gm_diag_scratch_size(int npos) { return (long long)DG_GRID * 8 + (npos > 0 ? npos : 0); }

extern "C" int gm_energy_balance(const gm_energy_args* g, const gm_props* p, void* stream) {
  if (!g || !p || !g->T0 || !g->T1 || !g->out || !g->scratch) return GM_ERR_ARG;
  if (g->nodes[0] < 3 || g->nodes[1] < 3 || g->nodes[2] < 2 || g->ne_planes < 1 || g->ne_planes > g->nodes[2] - 1)
    return GM_ERR_ARG;
  if (g->npos < 0 || (g->npos > 0 && !g->rows) || !(g->interval >= 0)) return GM_ERR_ARG;
  if (g->dtype != GM_F32 && g->dtype != GM_F64) return GM_ERR_ARG;
  if (gm_diag_scratch_size(g->npos) > g->scratch_cap) return GM_ERR_TOO_LARGE;
  EnergyK a;
  a.nx = g->nodes[0];
  a.ny = g->nodes[1];
  a.nz = g->nodes[2];
  a.ne_planes = g->ne_planes;
  a.dtype = g->dtype;
  a.hx = g->h[0];
  a.hy = g->h[1];
  a.hz = g->h[2];
  a.T0 = g->T0;
  a.T1 = g->T1;
  a.ph = g->ph;
  a.substrate = g->substrate;
  for (int m = 0; m < 8; ++m) {
    const int mx = m & 1, my = (m >> 1) & 1, mz = (m >> 2) & 1;
    const double Mx = mx ? a.hx / 6 : a.hx / 2, My = my ? a.hy / 6 : a.hy / 2, Mz = mz ? a.hz / 6 : a.hz / 2;
    const double Kx = mx ? 2 / a.hx : 0, Ky = my ? 2 / a.hy : 0, Kz = mz ? 2 / a.hz : 0;
    a.lam[m] = (Kx * My * Mz + Mx * Ky * Mz + Mx * My * Kz) / 8.0;
  }
  a.wvol = a.hx * a.hy * a.hz / 8.0;
  a.w2 = a.hx * a.hy / 4.0;
  a.p = make_props<double>(*p);
  cudaStream_t st = (cudaStream_t)stream;
  const long long ne = (long long)(a.nx - 1) * (a.ny - 1) * a.ne_planes;
  const int nb = dgrid(ne);
  double* part = g->scratch;
  double* spart = g->scratch + (long long)DG_GRID * 8;
  if (g->dtype == GM_F32)
    energy_elem_kernel<float><<<nb, DG_BLOCK, 0, st>>>(a, part);
  else
    energy_elem_kernel<double><<<nb, DG_BLOCK, 0, st>>>(a, part);
  if (cudaGetLastError() != cudaSuccess) return GM_ERR_LAUNCH;
  if (g->npos > 0) {
    const double r = p->laser_radius, d = p->laser_depth;
    const double rc = 1.0 / (r * sqrt(M_PI)), dc = 1.0 / (d * sqrt(M_PI));
    const double src_c = 6.0 * sqrt(3.0) * p->laser_eta * rc * rc * dc * a.wvol;
    energy_source_kernel<<<g->npos, DG_BLOCK, 0, st>>>(a.nx, a.ny, a.nz, a.ne_planes, g->origin[0], g->origin[1],
                                                      g->origin[2], a.hx, a.hy, a.hz, g->rows, 1.0 / (r * r),
                                                      1.0 / (d * d), src_c, spart);
    if (cudaGetLastError() != cudaSuccess) return GM_ERR_LAUNCH;
  }
  energy_final_kernel<<<1, 32, 0, st>>>(part, nb, spart, g->npos, g->interval, g->out);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_melt_pool(const gm_meltpool_args* g, void* stream) {
  if (!g || !g->T || !g->out || !g->scratch) return GM_ERR_ARG;
  if (g->nodes[0] < 1 || g->nodes[1] < 1 || g->nodes[2] < 1) return GM_ERR_ARG;
  if (gm_diag_scratch_size(0) > g->scratch_cap) return GM_ERR_TOO_LARGE;
  const long long n = (long long)g->nodes[0] * g->nodes[1] * g->nodes[2];
  const int nb = dgrid(n);
  cudaStream_t st = (cudaStream_t)stream;
  if (g->dtype == GM_F32)
    meltpool_kernel<float><<<nb, DG_BLOCK, 0, st>>>(g->nodes[0], g->nodes[1], g->nodes[2], g->origin[0],
                                                    g->origin[1], g->origin[2], g->h[0], g->h[1], g->h[2], g->T,
                                                    g->iso, g->scratch);
  else if (g->dtype == GM_F64)
    meltpool_kernel<double><<<nb, DG_BLOCK, 0, st>>>(g->nodes[0], g->nodes[1], g->nodes[2], g->origin[0],
                                                     g->origin[1], g->origin[2], g->h[0], g->h[1], g->h[2], g->T,
                                                     g->iso, g->scratch);
  else
    return GM_ERR_ARG;
  if (cudaGetLastError() != cudaSuccess) return GM_ERR_LAUNCH;
  meltpool_final_kernel<<<1, 32, 0, st>>>(g->scratch, nb, g->out);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_field_error(int dtype_a, const void* a, int dtype_b, const void* b, long long n, double* scratch,
                              long long scratch_cap, double* out, void* stream) {
  if (!a || !b || !scratch || !out || n < 0) return GM_ERR_ARG;
  if (gm_diag_scratch_size(0) > scratch_cap) return GM_ERR_TOO_LARGE;
  const int nb = dgrid(n);
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype_a == GM_F32 && dtype_b == GM_F64)
    field_err_kernel<float, double><<<nb, DG_BLOCK, 0, st>>>(n, a, b, scratch);
  else if (dtype_a == GM_F32 && dtype_b == GM_F32)
    field_err_kernel<float, float><<<nb, DG_BLOCK, 0, st>>>(n, a, b, scratch);
  else if (dtype_a == GM_F64 && dtype_b == GM_F64)
    field_err_kernel<double, double><<<nb, DG_BLOCK, 0, st>>>(n, a, b, scratch);
  else if (dtype_a == GM_F64 && dtype_b == GM_F32)
    field_err_kernel<double, float><<<nb, DG_BLOCK, 0, st>>>(n, a, b, scratch);
  else
    return GM_ERR_ARG;
  if (cudaGetLastError() != cudaSuccess) return GM_ERR_LAUNCH;
  field_err_final_kernel<<<1, 32, 0, st>>>(scratch, nb, n, out);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}
