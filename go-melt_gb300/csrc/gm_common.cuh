// Shared device helpers for the GO-MELT GB300 kernels.
//
// Data layout (all levels): structured node grids, node-major with x fastest,
// node id = ix + iy*nx + iz*nx*ny; element (ex,ey,ez) has corner nodes
// (ex+ax, ey+ay, ez+az), a* in {0,1}.  This is the layout of the reference's
// convert2XYZ (go_melt/computeFunctions.py:645-689).
//
// Phase byte per node: bit0 = S1 (bulk/solidified), bit1 = S2 (liquid).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>
#include "gomelt.h"

namespace gm {

constexpr uint8_t PH_S1 = 1;
constexpr uint8_t PH_S2 = 2;

// Arithmetic whose rounding is fixed by the source: the compiler neither
// fuses these products and sums into multiply-adds nor splits the explicit
// multiply-adds, whichever kernel inlines them.  Kernels that must give the
// same bits as one another (the one-step, batched and multi-step Level-3
// kernels) write their stencil with these.
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float rfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double rfma(double a, double b, double c) { return __fma_rn(a, b, c); }

template <typename real>
struct Props {
  real k_powder, k_bulk_a0, k_bulk_a1, k_fluid;  // W/(mm K)  (already /1000)
  real cp_solid_a0, cp_solid_a1, cp_mushy, cp_fluid, rho;
  real T_amb, T_solidus, T_liquidus, T_boiling;
  real h_conv, sig_eps, evc, Lev, CM, CT, CP;  // surface model (reference units)
  real Ta4;                                      // T_amb^4
};

template <typename real>
inline Props<real> make_props(const gm_props& p) {
  Props<real> q;
  q.k_powder = (real)(p.k_powder / 1000.0);
  q.k_bulk_a0 = (real)(p.k_bulk_a0 / 1000.0);
  q.k_bulk_a1 = (real)(p.k_bulk_a1 / 1000.0);
  q.k_fluid = (real)(p.k_fluid / 1000.0);
  q.cp_solid_a0 = (real)p.cp_solid_a0;
  q.cp_solid_a1 = (real)p.cp_solid_a1;
  q.cp_mushy = (real)p.cp_mushy;
  q.cp_fluid = (real)p.cp_fluid;
  q.rho = (real)p.rho;
  q.T_amb = (real)p.T_amb;
  q.T_solidus = (real)p.T_solidus;
  q.T_liquidus = (real)p.T_liquidus;
  q.T_boiling = (real)p.T_boiling;
  q.h_conv = (real)p.h_conv;
  q.sig_eps = (real)(p.sigma_sb * p.emissivity);
  q.evc = (real)p.evc;
  q.Lev = (real)p.Lev;
  q.CM = (real)p.CM_coeff;
  q.CT = (real)p.CT_coeff;
  q.CP = (real)p.CP_coeff;
  q.Ta4 = (real)(p.T_amb * p.T_amb * p.T_amb * p.T_amb);
  return q;
}

// Phase update and material properties of one node
// (computeStateProperties, go_melt/computeFunctions.py:2567-2614):
//   S2 = T >= T_liquidus; S3 = T_solidus < T < T_liquidus;
//   S1 = (S1_old > 0.499) | S2, forced to 1 on substrate nodes;
//   k  = [(1-S1)(1-S2) k_p + S1(1-S2)(a1 T + a0) + S2 k_f] / 1000
//   rc = rho [(1-S2)(1-S3)(c1 T + c0) + S3 c_m + S2 c_f]
// The products of 0/1 flags select exactly one term, so a select chain gives
// the same value.
template <typename real>
__device__ __forceinline__ uint8_t node_props(const Props<real>& p, real T, uint8_t ph_old, bool substrate,
                                              real& k, real& rc) {
  const bool s2 = T >= p.T_liquidus;
  const bool s3 = (T > p.T_solidus) && (T < p.T_liquidus);
  const bool s1 = (ph_old & PH_S1) || s2 || substrate;
  if (s2) {
    k = p.k_fluid;
  } else if (s1) {
    k = p.k_bulk_a1 * T + p.k_bulk_a0;
  } else {
    k = p.k_powder;
  }
  real cp;
  if (s2) {
    cp = p.cp_fluid;
  } else if (s3) {
    cp = p.cp_mushy;
  } else {
    cp = p.cp_solid_a1 * T + p.cp_solid_a0;
  }
  rc = p.rho * cp;
  return (uint8_t)((s1 ? PH_S1 : 0) | (s2 ? PH_S2 : 0));
}

// Phase and properties with selects (same values as node_props).  Returns the
// new phase bits (bit0 S1, bit1 S2).
template <typename real>
__device__ __forceinline__ uint32_t node_props_sel(const Props<real>& p, real T, uint32_t ph_old, bool substrate,
                                                   real& k, real& rc) {
  const bool s2 = T >= p.T_liquidus;
  const bool s3 = (T > p.T_solidus) && (T < p.T_liquidus);
  const bool s1 = (ph_old & PH_S1) || s2 || substrate;
  const real kb = p.k_bulk_a1 * T + p.k_bulk_a0;
  const real cs = p.cp_solid_a1 * T + p.cp_solid_a0;
  k = s2 ? p.k_fluid : (s1 ? kb : p.k_powder);
  rc = p.rho * (s2 ? p.cp_fluid : (s3 ? p.cp_mushy : cs));
  return (s1 ? PH_S1 : 0u) | (s2 ? PH_S2 : 0u);
}

// One staged node (or one exchanged corner sum) as a single 16/32-byte
// shared-memory record.
template <typename real>
struct alignas(4 * sizeof(real)) V4 {
  real x, y, z, w;
};
// 8-point Hadamard butterflies over the corner values of a brick element
// (index x + 2y + 4z): forward (a, b) -> (a + b, b - a) per axis, inverse
// (a, b) -> (a - b, a + b); inverse(forward(v)) = 8 v.
template <typename real>
__device__ __forceinline__ void bfly_fwd(real v[8]) {
#pragma unroll
  for (int s = 1; s < 8; s <<= 1) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if ((i & s) == 0) {
        const real a = v[i], b = v[i + s];
        v[i] = a + b;
        v[i + s] = b - a;
      }
    }
  }
}

template <typename real>
__device__ __forceinline__ void bfly_inv(real v[8]) {
#pragma unroll
  for (int s = 1; s < 8; s <<= 1) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if ((i & s) == 0) {
        const real a = v[i], b = v[i + s];
        v[i] = a - b;
        v[i + s] = a + b;
      }
    }
  }
}

// 1-D source factor of node i: sum over the (up to two) elements touching the
// node and their two Gauss points of N_local * exp(-3 (xq - v)^2 / r^2).
// rel = origin - v (formed in double by the caller), so the Gauss-point
// offset rel + h*(e + (1 +- 1/sqrt3)/2) is small and exact enough in the
// kernel's precision.
template <typename real>
__device__ __forceinline__ real src_factor(int i, int n, real rel, real h, real inv_r2) {
  const real g0 = (real)0.21132486540518711775, g1 = (real)0.78867513459481288225;  // (1 -+ 1/sqrt3)/2
  real s = 0;
  for (int e = i - 1; e <= i; ++e) {
    if (e < 0 || e >= n - 1) continue;
    const real d0 = rfma(h, radd((real)e, g0), rel);
    const real d1 = rfma(h, radd((real)e, g1), rel);
    const real q0 = exp(rmul(rmul((real)-3 * d0, d0), inv_r2));
    const real q1 = exp(rmul(rmul((real)-3 * d1, d1), inv_r2));
    // node i is local node 0 of element e when i == e: weights (1-xi)/2 = g1 at xi=-1/sqrt3, g0 at +1/sqrt3
    s = radd(s, (i == e) ? rfma(g1, q0, rmul(g0, q1)) : rfma(g0, q0, rmul(g1, q1)));
  }
  return s;
}

// Flux into the top surface at one Gauss point [W/mm^2]
// (computeConvRadBC, go_melt/computeFunctions.py:2263-2290).
template <typename real>
__device__ __forceinline__ real surface_flux(const Props<real>& p, real Tq) {
  Tq = fmin(Tq, radd(p.T_boiling, (real)1000));
  const real T2 = rmul(Tq, Tq);
  real q = rfma(p.h_conv, rsub(p.T_amb, Tq), rmul(p.sig_eps, rfma(-T2, T2, p.Ta4)));
  if (p.evc != (real)0) {
    const real invT = (real)1 / Tq;
    const real E_pv = rfma(p.cp_fluid, rsub(Tq, p.T_amb), p.Lev);
    const real MolMot = sqrt(rmul(p.CM, invT));
    const real S = rmul(rmul(rmul(rmul(p.evc, p.CP), exp(rmul(-p.CT, rsub(invT, (real)1 / p.T_boiling)))), MolMot),
                        E_pv);
    q = rsub(q, S);
  }
  return rmul(q, (real)1e-6);
}

// Per-axis interpolation map: target index t -> source element e[t] with the
// two linear weights (w[2t], w[2t+1]) = ((x_{e+1}-x)/h, (x-x_e)/h).
template <typename real>
struct AxisMap {
  const int* e;
  const real* w;
};

template <typename real>
struct Map3 {
  AxisMap<real> ax[3];
  int src_nx, src_ny;  // source node strides
};

// Trilinear weights of the reference's compute3DN (:1361-1393) from per-axis
// weights, with the validity rule of interpolatePointsMatrix (:1100-1102):
// if any of the 8 weights leaves [-0.01, 1.01] all are zero, else they are
// clipped to [0, 1].  Returns the base node id; w8 in reference node order.
template <typename real>
__device__ __forceinline__ int map3_weights(const Map3<real>& m, int tx, int ty, int tz, real w8[8]) {
  const int ex = m.ax[0].e[tx], ey = m.ax[1].e[ty], ez = m.ax[2].e[tz];
  const real x0 = m.ax[0].w[2 * tx], x1 = m.ax[0].w[2 * tx + 1];
  const real y0 = m.ax[1].w[2 * ty], y1 = m.ax[1].w[2 * ty + 1];
  const real z0 = m.ax[2].w[2 * tz], z1 = m.ax[2].w[2 * tz + 1];
  w8[0] = x0 * y0 * z0;
  w8[1] = x1 * y0 * z0;
  w8[2] = x1 * y1 * z0;
  w8[3] = x0 * y1 * z0;
  w8[4] = x0 * y0 * z1;
  w8[5] = x1 * y0 * z1;
  w8[6] = x1 * y1 * z1;
  w8[7] = x0 * y1 * z1;
  bool ok = true;
#pragma unroll
  for (int i = 0; i < 8; ++i) ok = ok && (w8[i] >= (real)-1e-2) && (w8[i] <= (real)(1 + 1e-2));
#pragma unroll
  for (int i = 0; i < 8; ++i) w8[i] = ok ? fmin(fmax(w8[i], (real)0), (real)1) : (real)0;
  return ex + ey * m.src_nx + ez * m.src_nx * m.src_ny;
}

template <typename real>
__device__ __forceinline__ real map3_apply(const Map3<real>& m, int tx, int ty, int tz, const real* __restrict__ u) {
  real w8[8];
  const int b = map3_weights(m, tx, ty, tz, w8);
  const int sx = 1, sy = m.src_nx, sz = m.src_nx * m.src_ny;
  return w8[0] * u[b] + w8[1] * u[b + sx] + w8[2] * u[b + sx + sy] + w8[3] * u[b + sy] + w8[4] * u[b + sz] +
         w8[5] * u[b + sx + sz] + w8[6] * u[b + sx + sy + sz] + w8[7] * u[b + sy + sz];
}

template <typename real>
inline Map3<real> make_map3(const gm_map3& m) {
  Map3<real> r;
  for (int d = 0; d < 3; ++d) {
    r.ax[d].e = m.elem[d];
    r.ax[d].w = (const real*)m.w[d];
  }
  r.src_nx = m.src_nx;
  r.src_ny = m.src_ny;
  return r;
}

__host__ __device__ inline int cdiv(int a, int b) { return (a + b - 1) / b; }

// Programmatic dependent launch.  A kernel that starts with pdl_begin() lets
// the next kernel in the stream launch its CTAs early and then waits until
// the kernel before it has completed (its writes visible) before it touches
// any field.  Without a programmatic dependency both instructions are no-ops.
__device__ __forceinline__ void pdl_begin() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// Whether launches through launch_k on this thread carry the programmatic
// dependency (set by gm_subcycle for the launches of one call).
inline bool& pdl_mode() {
  static thread_local bool on = false;
  return on;
}

struct PdlScope {
  bool prev;
  explicit PdlScope(bool on) : prev(pdl_mode()) { pdl_mode() = on; }
  ~PdlScope() { pdl_mode() = prev; }
};

// Kernel launch on `st`, as a programmatic dependent when pdl_mode() is set
// (only for kernels that begin with pdl_begin()).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                            Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl_mode() ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace gm
