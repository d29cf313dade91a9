// Fused explicit level step (one forward-Euler step of one GO-MELT level).
//
// Replaces, for one level, the reference's sequence computeStateProperties ->
// computeSourcesL3 -> computeConvRadBC -> solveMatrixFreeFE -> substitute_Tbar
// -> assignBCs/assignBCsFine -> max(T, T_amb) (go_melt/computeFunctions.py
// :2567-2614, :2960-3012, :2207-2301, :582-642, :1848-1865, :1568-1620).
//
// Scheme (identical algebra to solveMatrixFreeFE):
//   T_new(i) = T(i) + [ sum_e R_e(i) + F(i) + Corr(i) ] / M(i)
//   R_e = -kbar_e * K_ref * T_e,  M(i) = sum_e wq * mean_e(rho c) / dt
// which equals (sum_e (diag(Me) - Ke) T_e + F + Corr) / sum_e Me.
// K_ref (the exact 2x2x2-Gauss hex8 stiffness of a brick) is diagonal in the
// 8-point Hadamard basis of the element's corner values, so K_ref*T_e is a
// forward butterfly, 7 scalings and a backward butterfly.
//
// Thread mapping: a CTA of TX x BY threads (a tile row is a warp or a
// half-warp) owns a TX x BY tile of element columns and marches up a range of
// node planes.  Node planes are staged in two shared-memory slots (T, k,
// rho*c, phase bits).  Element corner contributions are combined onto nodes
// without atomics: x-neighbours by shuffle, y-neighbours through shared
// memory, z-neighbours by a register carry from one plane to the next.  Each
// CTA writes (TX-1) x (BY-1) node columns.
#include <math.h>

#include <map>
#include <mutex>
#include <type_traits>
#include <vector>

#include "gm_common.cuh"
#include "gm_sep.cuh"

namespace gm {

template <typename real>
struct LevelK {
  int nx, ny, nz, ne_planes, zchunk;
  double ox, oy, oz, hx, hy, hz;
  const double* dt;
  const real* T_in;
  real* T_out;
  const uint8_t* ph_in;
  uint8_t* ph_out;
  long long substrate;
  const real* k_arr;
  const real* rc_arr;
  const real* F_full;
  const real* corr_full;
  const real* rhs_box;
  int box[6];
  const double* laser;
  int surface, bc_mode, inactive_amb, clamp;
  real face[5];
  const real* bc_new;
  const real* bc_old;
  real bc_alpha, bc_beta;
  Map3<real> bc_map;
  real* accum;
  real* max_accum;
  int* status;  // optional: GM_STATUS_BAD_T when a new value is non-finite or above 1e5 K
  real lam[8];  // Hadamard-mode eigenvalues of K_ref, divided by 8
  real wvol;    // hx*hy*hz/8
  real w2;      // hx*hy/4
  double inv_r2, inv_d2;
  double src_c;  // 6*sqrt(3)*eta * rc^2 * dc * wvol  (times P)
  Props<real> p;
  // separable form (constant k, rho*c), formed on the host in double:
  real rh[3];            // hx, hy, hz
  real rir2, rid2;       // 1/r^2, 1/d^2 of the laser
  real sa1, sb1, sb2;    // k hy hz / (36 hx), k hx hz / (36 hy), k hx hy / (36 hz)
  real smass;            // lumped mass of 8 elements times dt: hx hy hz rho c
  const real* src_tab;   // optional laser factors of this step: [nx] x (times the power), [ny] y, [nz] z
};

constexpr int ZMAX = 64;

// x/y butterfly of one face (4 corner values, index x + 2y): the first two
// stages of bfly_fwd, which act on each face separately.
template <typename real>
__device__ __forceinline__ void face_fwd(real v[4]) {
  real a = v[0], b = v[1];
  v[0] = a + b;
  v[1] = b - a;
  a = v[2];
  b = v[3];
  v[2] = a + b;
  v[3] = b - a;
  a = v[0];
  b = v[2];
  v[0] = a + b;
  v[2] = b - a;
  a = v[1];
  b = v[3];
  v[1] = a + b;
  v[3] = b - a;
}

template <typename real>
__device__ __forceinline__ real fast_div(real a, real b) {
  return a / b;
}
template <>
__device__ __forceinline__ float fast_div<float>(float a, float b) {
  return __fdividef(a, b);
}

__device__ __forceinline__ float bits_as_real(uint32_t u, float) { return __uint_as_float(u); }
__device__ __forceinline__ double bits_as_real(uint32_t u, double) { return __longlong_as_double((long long)u); }
__device__ __forceinline__ uint32_t real_bits(float r) { return __float_as_uint(r); }
__device__ __forceinline__ uint32_t real_bits(double r) { return (uint32_t)__double_as_longlong(r); }

// Feature flags of a level-step instantiation.  LF_GENERIC compiles every
// feature with run-time checks; the other combinations are the ones the
// subcycle orchestrator issues, with every check resolved at compile time.
enum : int {
  LF_LASER = 1 << 0,
  LF_BOX = 1 << 1,
  LF_FULL = 1 << 2,
  LF_KARR = 1 << 3,
  LF_ACCUM = 1 << 4,
  LF_SURF = 1 << 5,
  LF_CLAMP = 1 << 6,
  LF_INACT = 1 << 7,
  LF_BC1 = 1 << 8,
  LF_BC2 = 1 << 9,
  LF_BC3 = 1 << 10,
  LF_PHIN = 1 << 11,
  LF_PHOUT = 1 << 12,
  LF_CONST = 1 << 13,  // k and rho*c independent of phase and temperature
  LF_GENERIC = 1 << 20
};
constexpr int LF_L3 = LF_LASER | LF_SURF | LF_CLAMP | LF_BC3 | LF_PHIN | LF_PHOUT;  // Level-3 step
constexpr int LF_L3ACC = LF_L3 | LF_ACCUM;                                         // ... with melt time
constexpr int LF_L2 = LF_BOX | LF_SURF | LF_CLAMP | LF_BC3 | LF_PHIN | LF_PHOUT;   // Level-2 step
constexpr int LF_L1 = LF_BOX | LF_SURF | LF_CLAMP | LF_INACT | LF_BC1 | LF_PHIN;  // Level-1 step (phase kept)

// Pipeline per CTA (one barrier per node plane):
//   two shared-memory slots of staged node planes (T, k, rho*c, phase bits),
//   plane p in slot p&1; the loop is unrolled by two so that every slot
//   address is a compile-time offset.  Iteration ke reads the upper corners
//   (plane ke+1, slot (ke+1)&1), stages plane ke+2 (loaded into registers
//   during the previous iteration) into slot ke&1, whose plane ke was last
//   read before the previous barrier, issues the loads of plane ke+3 and of
//   the per-node inputs of node plane ke+1 (ring values, RHS box, melt time),
//   computes element plane ke, exchanges corner sums (shuffle in x, shared
//   memory in y), passes the barrier and finalizes node plane ke.  Lower-plane
//   corner values are carried in registers.  Staged phase bits: bit0/1 the
//   new S1/S2, bit2 the old S2 (melt-time reset).
template <typename real, int TX, int BY, int FL>
__device__ __forceinline__ void level_body(const LevelK<real>& a, int bx, int by, int bz) {
  constexpr bool G = (FL & LF_GENERIC) != 0;
  constexpr int PX = TX + 1, PY = BY + 1, NP = PX * PY, NT = TX * BY;
  static_assert(TX == 16 || TX == 32, "a tile row is a warp or a half-warp");
  constexpr int NSLOT = (NP + NT - 1) / NT;
  static_assert(NT <= NP, "slot 0 covers every thread");
  __shared__ V4<real> sN[2][NP];
  __shared__ V4<real> sX[2][BY][TX];
  __shared__ real sSx[PX], sSy[PY], sSz[ZMAX];

  const bool hLaser = G ? a.laser != nullptr : (FL & LF_LASER) != 0;
  const bool hBox = G ? a.rhs_box != nullptr : (FL & LF_BOX) != 0;
  const bool hF = G && a.F_full != nullptr;
  const bool hCorr = G && a.corr_full != nullptr;
  const bool hKarr = G && a.k_arr != nullptr;
  const bool hAcc = G ? a.accum != nullptr : (FL & LF_ACCUM) != 0;
  const bool hSurf = G ? a.surface != 0 : (FL & LF_SURF) != 0;
  const bool hClamp = G ? a.clamp != 0 : (FL & LF_CLAMP) != 0;
  const bool hInact = G ? a.inactive_amb != 0 : (FL & LF_INACT) != 0;
  const bool hPhin = G ? a.ph_in != nullptr : (FL & LF_PHIN) != 0;
  const bool hPhout = G ? a.ph_out != nullptr : (FL & LF_PHOUT) != 0;
  const int bcm = G ? a.bc_mode : ((FL & LF_BC1) ? 1 : ((FL & LF_BC3) ? 3 : 0));
  constexpr bool kConst = (FL & LF_CONST) != 0;  // element means of k and rho*c are the constants

  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const int nxy = nx * ny;
  const int X0 = bx * (TX - 1), Y0 = by * (BY - 1);
  const int Z0 = bz * a.zchunk, Z1 = min(nz, Z0 + a.zchunk);
  const int subs = a.substrate > (long long)nxy * nz ? nxy * nz : (int)a.substrate;
  const real dt = (real)(*a.dt);
  const real inv_dt = (real)1 / dt;
  const Props<real>& P = a.p;

  // ---- per-thread staging slots (constant over the plane loop) ----
  int sbase[NSLOT];  // node id of the slot in plane 0, or -1 outside the grid / tile
  real pfT[NSLOT];
  uint32_t pfP[NSLOT];
#pragma unroll
  for (int s = 0; s < NSLOT; ++s) {
    const int i = tid + s * NT;
    sbase[s] = -1;
    if (i < NP) {
      const int gx = X0 - 1 + i % PX, gy = Y0 - 1 + i / PX;
      if (gx >= 0 && gx < nx && gy >= 0 && gy < ny) sbase[s] = gx + gy * nx;
    }
  }
  auto fetch = [&](int pl) {
    const bool pin = pl >= 0 && pl < nz;
#pragma unroll
    for (int s = 0; s < NSLOT; ++s) {
      pfT[s] = 0;
      pfP[s] = 0;
      if (pin && sbase[s] >= 0) {
        const int id = sbase[s] + pl * nxy;
        pfT[s] = a.T_in[id];
        if (hPhin) pfP[s] = a.ph_in[id];
      }
    }
  };
  auto store = [&](int pl, int slot) {
    const bool pin = pl >= 0 && pl < nz;
#pragma unroll
    for (int s = 0; s < NSLOT; ++s) {
      const int i = tid + s * NT;
      if (s == 0 || i < NP) {
        real k = 0, c = 0;
        uint32_t ph = 0;
        if (pin && sbase[s] >= 0) {
          const int id = sbase[s] + pl * nxy;
          if (kConst) {  // phase bits only
            const bool s2 = pfT[s] >= P.T_liquidus;
            const bool s1 = (pfP[s] & PH_S1) || s2 || id < subs;
            ph = (s1 ? PH_S1 : 0u) | (s2 ? PH_S2 : 0u) | ((pfP[s] & PH_S2) << 1);
          } else {
            ph = node_props_sel(P, pfT[s], pfP[s], id < subs, k, c) | ((pfP[s] & PH_S2) << 1);
          }
          if (hKarr) {
            k = a.k_arr[id];
            c = a.rc_arr[id];
          }
        }
        V4<real> r;
        r.x = pfT[s];
        r.y = k;
        r.z = c;
        r.w = bits_as_real(ph, real(0));
        sN[slot][i] = r;
      }
    }
  };

  // ---- prologue: planes Z0-1 (slot 0), Z0 (slot 1) staged, plane Z0+1 in registers ----
  fetch(Z0 - 1);
  store(Z0 - 1, 0);
  fetch(Z0);
  store(Z0, 1);
  fetch(Z0 + 1);
  real srcP = 0;
  if (hLaser) {
    const real rx = (real)(a.ox - a.laser[0]), ry = (real)(a.oy - a.laser[1]), rz = (real)(a.oz - a.laser[2]);
    const real ir2 = (real)a.inv_r2, id2 = (real)a.inv_d2;
    srcP = (real)(a.src_c * a.laser[6]);
    for (int i = tid; i < PX + PY + (Z1 - Z0); i += NT) {
      if (i < PX) {
        const int g = X0 - 1 + i;
        sSx[i] = (g >= 0 && g < nx) ? src_factor<real>(g, nx, rx, (real)a.hx, ir2) : (real)0;
      } else if (i < PX + PY) {
        const int g = Y0 - 1 + (i - PX);
        sSy[i - PX] = (g >= 0 && g < ny) ? src_factor<real>(g, ny, ry, (real)a.hy, ir2) : (real)0;
      } else {
        const int g = Z0 + (i - PX - PY);
        sSz[i - PX - PY] = src_factor<real>(g, nz, rz, (real)a.hz, id2);
      }
    }
  }
  __syncthreads();

  const int ex = X0 - 1 + tx, ey = Y0 - 1 + ty;
  const bool col_ok = ex >= 0 && ex < nx - 1 && ey >= 0 && ey < ny - 1;
  const int ix = X0 + tx, iy = Y0 + ty;
  const bool out_col = tx < TX - 1 && ty < BY - 1 && ix < nx && iy < ny;
  const int top_el = a.ne_planes - 1;
  const real PQ = (real)0.78867513459481288225, MQ = (real)0.21132486540518711775;  // (1 +- 1/sqrt3)/2
  const int c00 = ty * PX + tx;  // slot offset of this element's (0,0) corner
  const int nid0 = ix + iy * nx;  // node id of this thread's output column in plane 0
  const bool ring_xy = ix == 0 || ix == nx - 1 || iy == 0 || iy == ny - 1;
  const bool box_xy = hBox && ix >= a.box[0] && ix < a.box[1] && iy >= a.box[2] && iy < a.box[3];
  const int box_off = box_xy ? (ix - a.box[0]) + (iy - a.box[2]) * (a.box[1] - a.box[0]) : 0;
  const int box_pl = (a.box[1] - a.box[0]) * (a.box[3] - a.box[2]);
  const real srcxy = (hLaser && out_col) ? srcP * sSx[tx + 1] * sSy[ty + 1] : (real)0;

  // carried lower face of the element plane (plane Z0-1, slot 0): its x/y
  // butterfly modes fl, the output node's temperature, sums of k and rho*c
  real fl[4], tl3, ksl = 0, csl = 0;
  uint32_t phl = 0;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const V4<real> r = sN[0][c00 + (c >> 1) * PX + (c & 1)];
    fl[c] = r.x;
    if (!kConst) {
      ksl += r.y;
      csl += r.z;
    }
    if (c == 3) phl = real_bits(r.w);
  }
  tl3 = fl[3];
  face_fwd(fl);
  __syncthreads();  // slot 0 is restaged in the first iteration

  // per-node inputs of the node plane finalized next (loaded one iteration ahead)
  real cRhs = 0, cBA = 0, cBB = 0, cAcc = 0, cMacc = 0, cF = 0, cC = 0;
  real carryU = 0, carryM = 0;

  auto body = [&](auto par, int ke) {
    constexpr int PAR = decltype(par)::value;  // (ke - Z0 + 1) & 1: plane p lives in slot (p - Z0 + 1) & 1
    real tu[4], ksu = 0, csu = 0;
    uint32_t phu = 0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const V4<real> r = sN[PAR ^ 1][c00 + (c >> 1) * PX + (c & 1)];
      tu[c] = r.x;
      if (!kConst) {
        ksu += r.y;
        csu += r.z;
      }
      if (c == 3) phu = real_bits(r.w);
    }
    store(ke + 2, PAR);
    fetch(ke + 3);

    // inputs of node plane ke+1 (used by the next iteration's finalize)
    real nRhs = 0, nBA = 0, nBB = 0, nAcc = 0, nMacc = 0, nF = 0, nC = 0;
    {
      const int pl = ke + 1;
      if (out_col && pl < Z1) {
        const int idn = nid0 + pl * nxy;
        if (box_xy && pl >= a.box[4] && pl < a.box[5]) nRhs = a.rhs_box[box_off + (pl - a.box[4]) * box_pl];
        if (bcm == 3 && (ring_xy || pl == 0)) {
          nBA = a.bc_new[idn];
          nBB = a.bc_old[idn];
        }
        if (hAcc) {
          nAcc = a.accum[idn];
          nMacc = a.max_accum[idn];
        }
        if (hF) nF = a.F_full[idn];
        if (hCorr) nC = a.corr_full[idn];
      }
    }

    // ---- element (ex, ey, ke) ----
    real fu[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) fu[c] = tu[c];
    face_fwd(fu);
    real R[8];
    real me = 0;
    const bool el_ok = col_ok && ke >= 0 && ke < a.ne_planes;
    if (el_ok) {
      // Hadamard modes: z butterfly of the two faces' x/y modes; mode 0 (the
      // constant) has eigenvalue 0
      R[0] = 0;
#pragma unroll
      for (int c = 1; c < 4; ++c) R[c] = fl[c] + fu[c];
#pragma unroll
      for (int c = 0; c < 4; ++c) R[4 + c] = fu[c] - fl[c];
      const real kbar = kConst ? P.k_fluid : (ksl + ksu) * (real)0.125;
      me = kConst ? a.wvol * (P.rho * P.cp_fluid) * inv_dt : a.wvol * ((csl + csu) * (real)0.125) * inv_dt;
#pragma unroll
      for (int m = 1; m < 8; ++m) R[m] *= a.lam[m] * kbar;
      bfly_inv(R);
      if (hSurf && ke == top_el) {
        // top face: 2x2 Gauss points on the face of the upper corners
#pragma unroll
        for (int qy = 0; qy < 2; ++qy)
#pragma unroll
          for (int qx = 0; qx < 2; ++qx) {
            const real px0 = qx ? MQ : PQ, px1 = qx ? PQ : MQ;
            const real py0 = qy ? MQ : PQ, py1 = qy ? PQ : MQ;
            const real Tq = px0 * py0 * tu[0] + px1 * py0 * tu[1] + px0 * py1 * tu[2] + px1 * py1 * tu[3];
            const real q = surface_flux(P, Tq) * a.w2;
            R[4] -= px0 * py0 * q;
            R[5] -= px1 * py0 * q;
            R[6] -= px0 * py1 * q;
            R[7] -= px1 * py1 * q;
          }
      }
    } else {
#pragma unroll
      for (int m = 0; m < 8; ++m) R[m] = 0;
    }

    // ---- corners -> nodes (R holds kbar*K*T minus sources): x by shuffle, y via smem ----
    real cx[4];  // index ay + 2*az
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int ay = j & 1, az = j >> 1;
      cx[j] = R[1 + 2 * ay + 4 * az] + __shfl_down_sync(0xffffffffu, R[2 * ay + 4 * az], 1, TX);
    }
    const real mx = me + __shfl_down_sync(0xffffffffu, me, 1, TX);
    {
      V4<real> w;
      w.x = cx[0];  // ay=0, lower
      w.y = cx[2];  // ay=0, upper
      w.z = mx;
      w.w = 0;
      sX[PAR][ty][tx] = w;
    }
    __syncthreads();
    real lowN = cx[1], upN = cx[3], mN = mx;
    if (ty + 1 < BY) {
      const V4<real> n = sX[PAR][ty + 1][tx];
      lowN += n.x;
      upN += n.y;
      mN += n.z;
    }

    // ---- finalize node plane ke ----
    if (ke >= Z0 && out_col) {
      const int id = nid0 + ke * nxy;
      real Rt = -(carryU + lowN);
      const real M = carryM + mN;
      const real Told = tl3;
      const uint32_t phn = phl;
      if (hLaser) Rt += srcxy * sSz[ke - Z0];
      if (hBox) Rt += cRhs;
      if (hF) Rt += cF;
      if (hCorr) Rt += cC;
      real Tn = Told + fast_div(Rt, M);
      if (hInact && ke > a.ne_planes) Tn = P.T_amb;
      if (bcm == 1) {
        if (iy == 0) Tn = a.face[2];
        if (iy == ny - 1) Tn = a.face[3];
        if (ix == 0) Tn = a.face[0];
        if (ix == nx - 1) Tn = a.face[1];
        if (ke == 0) Tn = a.face[4];
      } else if (bcm == 3) {
        if (ring_xy || ke == 0) Tn = a.bc_alpha * cBA + a.bc_beta * cBB;
      } else if (G && bcm == 2 && (ring_xy || ke == 0)) {
        real w8[8];
        const int b = map3_weights(a.bc_map, ix, iy, ke, w8);
        const int sx = 1, sy = a.bc_map.src_nx, sz = a.bc_map.src_nx * a.bc_map.src_ny;
        const int off[8] = {0, sx, sx + sy, sy, sz, sx + sz, sx + sy + sz, sy + sz};
        real v = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const real bc = a.bc_alpha * a.bc_new[b + off[j]] + a.bc_beta * a.bc_old[b + off[j]];
          v += w8[j] * bc;
        }
        Tn = v;
      }
      if (a.status && !(Tn <= (real)1e5)) atomicOr(a.status, GM_STATUS_BAD_T);
      if (hClamp) Tn = fmax(Tn, P.T_amb);
      a.T_out[id] = Tn;
      if (hPhout) a.ph_out[id] = (uint8_t)(phn & 3u);
      if (hAcc) {
        const bool prev2 = (phn & 4u) != 0;
        const bool s2 = (phn & PH_S2) != 0;
        const real racc = (s2 && !prev2) ? cAcc : (real)0;
        a.max_accum[id] = fmax(racc, cMacc);
        a.accum[id] = (cAcc + dt * (s2 ? (real)1 : (real)0)) - racc;
      }
    }
    carryU = upN;
    carryM = mN;
#pragma unroll
    for (int c = 0; c < 4; ++c) fl[c] = fu[c];
    tl3 = tu[3];
    ksl = ksu;
    csl = csu;
    phl = phu;
    cRhs = nRhs;
    cBA = nBA;
    cBB = nBB;
    cAcc = nAcc;
    cMacc = nMacc;
    cF = nF;
    cC = nC;
  };

  for (int ke = Z0 - 1; ke < Z1; ke += 2) {
    body(std::integral_constant<int, 0>(), ke);
    if (ke + 1 < Z1) body(std::integral_constant<int, 1>(), ke + 1);
  }
}

// Resident CTAs per SM: 4 for the FP32 constant-property variants (they fit
// 64 registers without spills), else 3 (FP32) or 2 (FP64).
template <typename real, int FL>
constexpr int level_min_blocks() {
  return sizeof(real) != 4 ? 2 : ((FL & LF_CONST) ? 4 : 3);
}

template <typename real, int TX, int BY, int FL>
__global__ void __launch_bounds__(TX * BY, level_min_blocks<real, FL>()) level_step_kernel(const LevelK<real> a) {
  level_body<real, TX, BY, FL>(a, blockIdx.x, blockIdx.y, blockIdx.z);
}

// ---------------------------------------------------------------------------
// Separable form of the level step for constant k and rho*c.
//
// With one conductivity and one heat capacity the element sum of
// solveMatrixFreeFE is the assembled brick operator, a tensor sum of 1-D
// operators over the active element box [0,nx-1) x [0,ny-1) x [0,ne_planes):
//   sum_e K_e T = k [Kx (x) My (x) Mz + Mx (x) Ky (x) Mz + Mx (x) My (x) Kz] T,
// 1-D stiffness K = (1/h)(-1, 2, -1) and consistent mass M = (h/6)(1, 4, 1)
// at a node with two elements, one-sided (1/h)(1, -1) and (h/6)(2, 1) at a
// node with one.  The lumped mass is (rho c / dt)(h^3/8) times the number of
// elements at the node (8 inside, 4 on the top plane).  Every node of the x/y
// ring and of the bottom plane is a Dirichlet node in the variants that use
// this kernel (bc_mode 1 and 3), so only the top plane needs the one-sided z
// operators.  Same algebra as level_body in a different order of summation.
//
// Thread mapping: a warp owns one x-tile of 30 node columns (lanes 1..30;
// lanes 0 and 31 are the x halo) and a strip of BYT consecutive y rows, and
// marches its CTA's z-chunk.  T planes p-1 .. p+3 of the strip and its two
// halo rows sit in a 6-deep register ring (plane p+3 is loaded while plane p
// is computed, so a load has two plane iterations to arrive); the phase and
// RHS-box inputs are loaded two planes ahead, the melt-time accumulators one
// plane ahead and only at liquid nodes.  z and y stencils are register
// arithmetic and the x stencil takes the neighbouring lanes' partial sums by
// shuffles, so warps never wait on one another.  The marching chunks cover
// node planes 1 .. ntop-1 (and the inactive planes above ntop); the top plane
// ntop (one-sided z operators, surface flux) is computed by a z-slice of its
// own, so the marching loop carries no top-plane case.  The Dirichlet nodes
// (x/y ring, bottom plane) are written by the last z-slice of CTAs, which does
// no stencil work: the marching warps neither load ring values nor store ring
// nodes.  The laser's 1-D source factors come from a table of the step
// (gm_fine_source_tables) or are evaluated per lane in the prologue.
// ---------------------------------------------------------------------------
constexpr int SEP_TILE = 30;  // output node columns of a warp
constexpr int SEP_ZMAX = 32;  // planes a CTA marches (one z source factor a lane)

// Node planes [1, sep_march_end) are marched in z-chunks; plane ntop (the top
// of the active element planes: one-sided z operators, surface flux) has a
// z-slice of CTAs of its own, and plane 0 is Dirichlet.  With inactive planes
// above ntop (reset to T_amb) the march runs to nz and passes over ntop.
__host__ __device__ inline int sep_march_end(int nz, int ntop, bool inact) {
  return inact && ntop < nz - 1 ? nz : ntop;
}
// z-slices of a separable launch: the marching chunks, then the top-plane
// slice, then the Dirichlet slice
__host__ __device__ inline int sep_march_chunks(int nz, int ntop, bool inact, int zc) {
  const int mz = sep_march_end(nz, ntop, inact);
  return mz > 1 ? cdiv(mz - 1, zc) : 0;
}

template <typename real, int BYT>
constexpr int sep_min_blocks() {
  // 256-thread CTAs: 64, 85 or 128 registers a thread
  return sizeof(real) != 4 ? 2 : (BYT == 1 ? 4 : (BYT == 2 ? 3 : 2));
}

// One CTA of the separable step: x-tile bx, strip group by, z-chunk bz of a
// (gx, gy, ring_z + 1) grid; z-slice ring_z - 1 is the top plane and ring_z
// the Dirichlet slice.
template <typename real, int BYT, int FL>
__device__ __forceinline__ void sep_body(const LevelK<real>& a, int bx, int by, int bz, int gx, int gy,
                                         int ring_z) {
  constexpr int RY = BYT + 2;  // strip rows with the two y halo rows
  constexpr unsigned FULL = 0xffffffffu;
  constexpr bool hLaser = (FL & LF_LASER) != 0;
  constexpr bool hBox = (FL & LF_BOX) != 0;
  constexpr bool hAcc = (FL & LF_ACCUM) != 0;
  constexpr bool hSurf = (FL & LF_SURF) != 0;
  constexpr bool hClamp = (FL & LF_CLAMP) != 0;
  constexpr bool hInact = (FL & LF_INACT) != 0;
  constexpr bool hPhout = (FL & LF_PHOUT) != 0;
  constexpr bool needPh = hPhout || hAcc;
  constexpr int bcm = (FL & LF_BC1) ? 1 : 3;
  static_assert((FL & LF_CONST) && !(FL & (LF_GENERIC | LF_KARR | LF_FULL | LF_BC2)), "constant-property variants");

  const int nx = a.nx, ny = a.ny, nz = a.nz, nxy = nx * ny;
  const int lane = threadIdx.x & 31;
  const int x = bx * SEP_TILE - 1 + lane;
  const int y0 = (by * (blockDim.x >> 5) + (threadIdx.x >> 5)) * BYT;
  const int ntop = a.ne_planes;
  const Props<real>& P = a.p;
  // Programmatic dependent launch: the next kernel in the stream may start its
  // CTAs now; they wait (griddepcontrol.wait) for this grid before touching
  // its fields.  Without a programmatic dependency both are no-ops.
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  // double-precision inputs converted once per CTA: dt and the laser's offsets
  // from the window origin and power factor (rx, ry, rz, srcP)
  __shared__ real s_in[5];
  if (threadIdx.x == 0) {
    s_in[0] = (real)(*a.dt);
    if (hLaser && !a.src_tab) {
      s_in[1] = (real)(a.ox - a.laser[0]);
      s_in[2] = (real)(a.oy - a.laser[1]);
      s_in[3] = (real)(a.oz - a.laser[2]);
      s_in[4] = (real)(a.src_c * a.laser[6]);
    }
  }
  __syncthreads();
  const real dt = s_in[0];
  const int subs = a.substrate > (long long)nxy * nz ? nxy * nz : (int)a.substrate;
  const bool xin = x >= 0 && x < nx;
  const bool out_x = lane >= 1 && lane <= SEP_TILE && x < nx;
  const bool ring_x = x == 0 || x == nx - 1;

  // New phase, output and melt time of node id (old temperature Told, phase
  // byte ph).  The melt-time update (acc + dt S2 - reset acc, max(reset acc,
  // macc)) leaves a node that is not liquid unchanged (macc >= 0), so the
  // accumulators are read (cAcc, cMacc) and written at liquid nodes only.
  bool bad = false;  // a new value non-finite or above 1e5 K (before the clamp)
  auto report = [&]() {
    if (bad && a.status) atomicOr(a.status, GM_STATUS_BAD_T);
  };
  auto finish = [&](int id, real Tn, real Told, uint32_t ph, real cAcc, real cMacc) {
    bad = bad || !(Tn <= (real)1e5);
    if (hClamp) Tn = fmax(Tn, P.T_amb);
    a.T_out[id] = Tn;
    if (needPh) {
      const bool s2 = Told >= P.T_liquidus;
      const bool s1 = (ph & PH_S1) || s2 || id < subs;
      if (hPhout) a.ph_out[id] = (uint8_t)((s1 ? PH_S1 : 0u) | (s2 ? PH_S2 : 0u));
      if (hAcc && s2) {
        const bool prev2 = (ph & PH_S2) != 0;
        const real racc = prev2 ? (real)0 : cAcc;
        a.max_accum[id] = fmax(racc, cMacc);
        a.accum[id] = rsub(radd(cAcc, dt), racc);
      }
    }
  };

  if (bz == ring_z) {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    // ---- Dirichlet nodes, spread over the threads of this slice: the bottom
    // plane, then the x/y ring of planes 1..nz-1 (perimeter order y0, y1, x0, x1) ----
    // 32-bit enumeration: nring <= nx ny nz < 2^31 (node ids are 32-bit), and
    // an unsigned k + stride stays below 2^32
    const int perim = 2 * nx + 2 * (ny - 2);
    const unsigned nring = (unsigned)(nxy + (nz - 1) * perim);
    const long long t0 = ((long long)by * gx + bx) * blockDim.x + threadIdx.x;
    if (t0 >= nring) return;
    const unsigned nthr = (unsigned)min((long long)gx * gy * blockDim.x, (long long)nring);
#pragma unroll 4
    for (unsigned k = (unsigned)t0; k < nring; k += nthr) {
      int rx, ry, rp;
      if (k < (unsigned)nxy) {
        rp = 0;
        rx = (int)(k % (unsigned)nx);
        ry = (int)(k / (unsigned)nx);
      } else {
        const unsigned kk = k - (unsigned)nxy;
        rp = 1 + (int)(kk / (unsigned)perim);
        const int j = (int)(kk % (unsigned)perim);
        if (j < nx) {
          rx = j;
          ry = 0;
        } else if (j < 2 * nx) {
          rx = j - nx;
          ry = ny - 1;
        } else if (j < 2 * nx + ny - 2) {
          rx = 0;
          ry = 1 + j - 2 * nx;
        } else {
          rx = nx - 1;
          ry = 1 + j - 2 * nx - (ny - 2);
        }
      }
      const int id = rx + ry * nx + rp * nxy;
      real Tn;
      if (bcm == 1) {
        Tn = a.face[4];
        if (rp > 0) {
          Tn = (ry == 0) ? a.face[2] : a.face[3];
          if (rx == 0) Tn = a.face[0];
          if (rx == nx - 1) Tn = a.face[1];
        }
      } else {
        Tn = rfma(a.bc_alpha, a.bc_new[id], rmul(a.bc_beta, a.bc_old[id]));
      }
      const real Told = needPh ? a.T_in[id] : (real)0;
      const bool liq = hAcc && Told >= P.T_liquidus;
      finish(id, Tn, Told, needPh ? (uint32_t)a.ph_in[id] : 0u, liq ? a.accum[id] : (real)0,
             liq ? a.max_accum[id] : (real)0);
    }
    report();
    return;
  }

  // z-slice ring_z - 1 computes the top plane, the others march their chunk
  const bool top_slice = bz == ring_z - 1;
  if (top_slice && (ntop < 1 || ntop >= nz)) return;
  const int Z0 = top_slice ? ntop : 1 + bz * a.zchunk;
  const int Z1 = top_slice ? ntop + 1 : min(sep_march_end(nz, ntop, hInact), Z0 + a.zchunk);
  // stencil constants: A = a1 (Zm- + 4 Zm + Zm+), B = b1 Ky(Zm) + b2 My(Zk)
  const real a1 = a.sa1, b1 = a.sb1, b2 = a.sb2;
  const real minv = dt / a.smass;  // 1 / (8 elements' lumped mass)

  // laser: x factor times the rows' y factors; lane l keeps the z factor of
  // plane Z0 + l.
  real sxy[BYT], szl = 0;
  if (hLaser && a.src_tab) {  // the step's factors, tabulated before the subcycle (fine_source_tables)
    const real* tb = a.src_tab;
    const real sx = xin ? tb[x] : (real)0;
    const real syl = (lane < BYT && y0 + lane < ny) ? tb[nx + y0 + lane] : (real)0;
#pragma unroll
    for (int r = 0; r < BYT; ++r) sxy[r] = rmul(sx, __shfl_sync(FULL, syl, r));
    if (Z0 + lane < Z1) szl = tb[nx + ny + Z0 + lane];
  } else if (hLaser) {
    const real rx = s_in[1], ry = s_in[2], rz = s_in[3], srcP = s_in[4];
    const real sx = xin ? rmul(srcP, src_factor<real>(x, nx, rx, a.rh[0], a.rir2)) : (real)0;
    // lane r < BYT evaluates the y factor of row y0 + r for the whole warp
    const real syl =
        (lane < BYT && y0 + lane < ny) ? src_factor<real>(y0 + lane, ny, ry, a.rh[1], a.rir2) : (real)0;
#pragma unroll
    for (int r = 0; r < BYT; ++r) sxy[r] = rmul(sx, __shfl_sync(FULL, syl, r));
    if (Z0 + lane < Z1) szl = src_factor<real>(Z0 + lane, nz, rz, a.rh[2], a.rid2);
  }
  // every read and write of a field comes after the preceding grid completed
  asm volatile("griddepcontrol.wait;" ::: "memory");

  int box_w = 0, box_pl = 0;
  bool box_x = false;
  if (hBox) {
    box_w = a.box[1] - a.box[0];
    box_pl = box_w * (a.box[3] - a.box[2]);
    box_x = x >= a.box[0] && x < a.box[1];
  }
  // rows whose nodes this warp writes (not on the y ring, inside the grid)
  bool row_out[BYT];
#pragma unroll
  for (int r = 0; r < BYT; ++r) row_out[r] = out_x && !ring_x && y0 + r > 0 && y0 + r < ny - 1;

  real Tr[6][RY];
  const real* Tcol = a.T_in + (x + (y0 - 1) * nx);  // strip row 0 of plane 0 (dereferenced only inside the grid)
  auto load_plane = [&](real(&dst)[RY], int pl) {
    const bool ok = xin && pl >= 0 && pl < nz;
#pragma unroll
    for (int i = 0; i < RY; ++i) {
      const int y = y0 - 1 + i;
      dst[i] = (ok && y >= 0 && y < ny) ? Tcol[i * nx + pl * nxy] : (real)0;
    }
  };
  // per-node inputs of one output plane, loaded two planes ahead
  uint32_t nph[3][BYT];
  real nrhs[3][BYT];
  auto prefetch = [&](auto slot_c, int pl) {
    constexpr int S = decltype(slot_c)::value;
#pragma unroll
    for (int r = 0; r < BYT; ++r) {
      const int y = y0 + r;
      const bool ok = row_out[r] && pl < Z1;
      const int id = x + y * nx + pl * nxy;
      nph[S][r] = 0;
      nrhs[S][r] = 0;
      if (ok) {
        if (needPh) nph[S][r] = a.ph_in[id];
        if (hBox && box_x && y >= a.box[2] && y < a.box[3] && pl >= a.box[4] && pl < a.box[5])
          nrhs[S][r] = a.rhs_box[(x - a.box[0]) + (y - a.box[2]) * box_w + (pl - a.box[4]) * box_pl];
      }
    }
  };
  // melt-time accumulators of the liquid nodes of plane pl (T at the step
  // start in Tc), loaded one plane ahead; warps without liquid nodes skip it
  real nacc[2][BYT], nmac[2][BYT];
  auto prefetch_acc = [&](auto slot_c, int pl, const RegCol<real, BYT> Tc) {
    constexpr int S = decltype(slot_c)::value;
    bool liq[BYT], any = false;
#pragma unroll
    for (int r = 0; r < BYT; ++r) {
      liq[r] = row_out[r] && pl < Z1 && Tc.v[r] >= P.T_liquidus;
      any = any || liq[r];
      nacc[S][r] = nmac[S][r] = 0;
    }
    if (__any_sync(FULL, any)) {
#pragma unroll
      for (int r = 0; r < BYT; ++r)
        if (liq[r]) {
          const int id = x + (y0 + r) * nx + pl * nxy;
          nacc[S][r] = a.accum[id];
          nmac[S][r] = a.max_accum[id];
        }
    }
  };

  // the output rows of a strip column (strip rows 1..BYT)
  auto rows_of = [&](const real* c) {
    RegCol<real, BYT> o;
#pragma unroll
    for (int r = 0; r < BYT; ++r) o.v[r] = c[r + 1];
    return o;
  };
  // register arrays passed by value to plane_out
  auto strip_of = [&](const real* c) {
    RegCol<real, RY> o;
#pragma unroll
    for (int i = 0; i < RY; ++i) o.v[i] = c[i];
    return o;
  };
  auto node_of = [&](const real* c) {
    RegCol<real, BYT> o;
#pragma unroll
    for (int r = 0; r < BYT; ++r) o.v[r] = c[r];
    return o;
  };
  auto phase_of = [&](const uint32_t* c) {
    RegCol<uint32_t, BYT> o;
#pragma unroll
    for (int r = 0; r < BYT; ++r) o.v[r] = c[r];
    return o;
  };

  // New values of the strip's nodes of plane p from T planes p-1, p, p+1
  // (Tm, T0, Tp; Tp unused on the top plane) and the plane's per-node inputs.
  // TOP: one-sided z operators, the lumped mass of 4 elements, surface flux.
  auto plane_out = [&](auto top_c, int p, const RegCol<real, RY> Tm, const RegCol<real, RY> T0,
                       const RegCol<real, RY> Tp, const RegCol<real, BYT> surf, real sz,
                       const RegCol<uint32_t, BYT> ph, const RegCol<real, BYT> rhs, const RegCol<real, BYT> acc,
                       const RegCol<real, BYT> mac) {
    constexpr bool TOP = decltype(top_c)::value;
    // ---- z and y stencils in registers, x stencil by shuffles ----
    real Zm[RY], Zk[RY];
#pragma unroll
    for (int i = 0; i < RY; ++i) {
      if (TOP) {
        Zm[i] = rfma((real)2, T0.v[i], Tm.v[i]);
        Zk[i] = rsub(T0.v[i], Tm.v[i]);
      } else {
        const real s = radd(Tm.v[i], Tp.v[i]);
        Zm[i] = rfma((real)4, T0.v[i], s);
        Zk[i] = rfma((real)2, T0.v[i], -s);
      }
    }
    const real mi = TOP ? (real)2 * minv : minv;
#pragma unroll
    for (int r = 0; r < BYT; ++r) {
      const int i = r + 1;
      const real u = radd(Zm[i - 1], Zm[i + 1]);
      const real w = radd(Zk[i - 1], Zk[i + 1]);
      const real A = rmul(a1, rfma((real)4, Zm[i], u));
      const real B = rfma(b1, rfma((real)2, Zm[i], -u), rmul(b2, rfma((real)4, Zk[i], w)));
      // x stencil: (2A - A(x-1) - A(x+1)) + (B(x-1) + 4B + B(x+1)) = 2A + 4B + D(x-1) + D(x+1), D = B - A
      const real D = rsub(B, A);
      const real Dl = __shfl_up_sync(FULL, D, 1), Dr = __shfl_down_sync(FULL, D, 1);
      if (!row_out[r] || (!TOP && hInact && p == ntop)) continue;
      const real KT = radd(rfma((real)2, A, rmul((real)4, B)), radd(Dl, Dr));
      const real Told = T0.v[i];
      real Rt = -KT;
      if (hLaser) Rt = rfma(sxy[r], sz, Rt);
      if (hBox) Rt = radd(Rt, rhs.v[r]);
      if (TOP && hSurf) Rt = radd(Rt, surf.v[r]);
      real Tn = rfma(Rt, mi, Told);
      if (!TOP && hInact && p > ntop) Tn = P.T_amb;
      finish(x + (y0 + r) * nx + p * nxy, Tn, Told, ph.v[r], acc.v[r], mac.v[r]);
    }
  };

  if (top_slice) {
    real Tm[RY], T0[RY], surf[BYT];
    load_plane(Tm, ntop - 1);
    load_plane(T0, ntop);
    prefetch(std::integral_constant<int, 0>(), ntop);
    if (hAcc) prefetch_acc(std::integral_constant<int, 0>(), ntop, rows_of(T0));
#pragma unroll
    for (int r = 0; r < BYT; ++r) surf[r] = 0;
    if (hSurf) {  // convection / radiation / evaporation on the faces of element plane ntop-1
      RegCol<real, RY> col;
#pragma unroll
      for (int i = 0; i < RY; ++i) col.v[i] = T0[i];
      const RegCol<real, BYT> sf = sep_surface<real, BYT>(P, a.w2, x, nx, y0, ny, col);
#pragma unroll
      for (int r = 0; r < BYT; ++r) surf[r] = sf.v[r];
    }
    const real sz = hLaser ? __shfl_sync(FULL, szl, 0) : (real)0;
    plane_out(std::true_type(), ntop, strip_of(Tm), strip_of(T0), strip_of(T0), node_of(surf), sz, phase_of(nph[0]),
              node_of(nrhs[0]), node_of(nacc[0]), node_of(nmac[0]));
    report();
    return;
  }

  load_plane(Tr[0], Z0 - 1);
  load_plane(Tr[1], Z0);
  load_plane(Tr[2], Z0 + 1);
  load_plane(Tr[3], Z0 + 2);
  prefetch(std::integral_constant<int, 0>(), Z0);
  prefetch(std::integral_constant<int, 1>(), Z0 + 1);
  if (hAcc) prefetch_acc(std::integral_constant<int, 0>(), Z0, rows_of(Tr[1]));

  // plane q lives in T slot (q - Z0 + 1) % 6 and per-node slot (q - Z0) % 3;
  // iteration p issues the loads of plane p + 3 and the inputs of plane p + 2
  auto body = [&](auto par, int p) {
    constexpr int PAR = decltype(par)::value;
    constexpr int NB = PAR % 3;  // per-node input slot of plane p
    real(&Tm)[RY] = Tr[PAR % 6];
    real(&T0)[RY] = Tr[(PAR + 1) % 6];
    real(&Tp)[RY] = Tr[(PAR + 2) % 6];
    if (p + 3 <= Z1) load_plane(Tr[(PAR + 4) % 6], p + 3);
    prefetch(std::integral_constant<int, (PAR + 2) % 3>(), p + 2);
    if (hAcc) prefetch_acc(std::integral_constant<int, (PAR + 1) & 1>(), p + 1, rows_of(Tp));
    const real sz = hLaser ? __shfl_sync(FULL, szl, p - Z0) : (real)0;
    // the surface-flux column is read on the top plane only: any column serves here
    plane_out(std::false_type(), p, strip_of(Tm), strip_of(T0), strip_of(Tp), node_of(nrhs[NB]), sz, phase_of(nph[NB]),
              node_of(nrhs[NB]), node_of(nacc[PAR & 1]), node_of(nmac[PAR & 1]));
  };

  for (int p = Z0; p < Z1; p += 6) {
    body(std::integral_constant<int, 0>(), p);
    if (p + 1 < Z1) body(std::integral_constant<int, 1>(), p + 1);
    if (p + 2 < Z1) body(std::integral_constant<int, 2>(), p + 2);
    if (p + 3 < Z1) body(std::integral_constant<int, 3>(), p + 3);
    if (p + 4 < Z1) body(std::integral_constant<int, 4>(), p + 4);
    if (p + 5 < Z1) body(std::integral_constant<int, 5>(), p + 5);
  }
  report();
}

template <typename real, int BYT, int FL>
__global__ void __launch_bounds__(256, sep_min_blocks<real, BYT>()) level_sep_kernel(const LevelK<real> a) {
  sep_body<real, BYT, FL>(a, blockIdx.x, blockIdx.y, blockIdx.z, gridDim.x, gridDim.y, gridDim.z - 1);
}

// Many windows in one launch: instance b owns the linear CTAs
// [first[b], first[b+1]) of the grid, laid out (bx, by, bz) with bx fastest
// over its own (gx, gy, z-chunks + top and Dirichlet slices) grid; its parameters are
// read from tab[b] into shared memory once per CTA.
template <typename real, int BYT, int FL>
__global__ void __launch_bounds__(256, sep_min_blocks<real, BYT>())
    level_sep_batched_kernel(const LevelK<real>* __restrict__ tab, const int* __restrict__ first, int nb) {
  __shared__ LevelK<real> sa;
  __shared__ int sb[6];
  if (threadIdx.x == 0) {
    const int blk = blockIdx.x;
    int lo = 0, hi = nb - 1;
    while (lo < hi) {  // last instance with first[b] <= blk
      const int mid = (lo + hi + 1) >> 1;
      if (first[mid] <= blk)
        lo = mid;
      else
        hi = mid - 1;
    }
    sa = tab[lo];
    const int local = blk - first[lo];
    const int gx = cdiv(sa.nx, SEP_TILE), gy = cdiv(sa.ny, (int)(blockDim.x >> 5) * BYT);
    sb[0] = local % gx;
    sb[1] = (local / gx) % gy;
    sb[2] = local / (gx * gy);
    sb[3] = gx;
    sb[4] = gy;
    sb[5] = sep_march_chunks(sa.nz, sa.ne_planes, (FL & LF_INACT) != 0, sa.zchunk) + 1;  // the Dirichlet slice
  }
  __syncthreads();
  sep_body<real, BYT, FL>(sa, sb[0], sb[1], sb[2], sb[3], sb[4], sb[5]);
}

// Many level windows (instances of uneven sizes) in one launch: instance b
// owns the linear blocks [first[b], first[b+1]) of the grid, laid out
// (bx, by, bz) with bx fastest over its own tiles; its parameters are read
// from tab[b] into shared memory once per block.
template <typename real, int TX, int BY, int FL>
__global__ void __launch_bounds__(TX * BY, sizeof(real) == 4 ? 3 : 2)
    level_step_batched_kernel(const LevelK<real>* __restrict__ tab, const int* __restrict__ first, int nb) {
  __shared__ LevelK<real> sa;
  __shared__ int sb[3];
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    const int blk = blockIdx.x;
    int lo = 0, hi = nb - 1;
    while (lo < hi) {  // last instance with first[b] <= blk
      const int mid = (lo + hi + 1) >> 1;
      if (first[mid] <= blk)
        lo = mid;
      else
        hi = mid - 1;
    }
    sa = tab[lo];
    const int local = blk - first[lo];
    const int gx = cdiv(sa.nx, TX - 1), gy = cdiv(sa.ny, BY - 1);
    sb[0] = local % gx;
    sb[1] = (local / gx) % gy;
    sb[2] = local / (gx * gy);
  }
  __syncthreads();
  level_body<real, TX, BY, FL>(sa, sb[0], sb[1], sb[2]);
}

// Tile of one CTA: 32 x 8 element columns (31 x 7 output node columns).
// Measured on the 161 x 161 x 41-node Level-3 window against 16 x 16 tiles
// over z-chunks of 4..41 planes: 17.1 us (32 x 8, 14 planes) vs 17.4 us
// (16 x 16, 12 planes) per launch.
constexpr int LT_X = 32, LT_Y = 8;

// Node planes per CTA when the caller does not choose.  The kernel is bound
// by instruction issue, so the time of a launch follows the busiest SM:
// (CTAs per SM) x (planes per CTA + 1 halo plane), divided by an issue
// efficiency that drops when fewer than three CTAs share an SM.  Among equal
// costs the smallest total work wins.
template <typename real, int TX, int BY, int FL>
static int auto_zchunk(int tiles_xy, int nz) {
  static int sms = 0, per = 0;
  if (sms == 0) {
    int dev = 0, n = 0, p = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p, level_step_kernel<real, TX, BY, FL>, TX * BY, 0);
    per = p > 0 ? p : 1;
    sms = n > 0 ? n : 152;
  }
  static const double eff[4] = {1.0, 0.55, 0.85, 1.0};
  int best = nz < ZMAX ? nz : ZMAX;
  double best_cost = -1;
  long long best_total = 0;
  for (int nch = cdiv(nz, ZMAX); nch <= nz; ++nch) {
    const int zc = cdiv(nz, nch);
    if (cdiv(nz, zc) != nch) continue;  // the same split as a smaller chunk count
    const long long ctas = (long long)tiles_xy * nch;
    const long long per_sm = (ctas + sms - 1) / sms;
    const long long res = per_sm < per ? per_sm : per;
    const double cost = (double)(per_sm * (zc + 1)) / eff[res < 3 ? res : 3];
    const long long total = ctas * (zc + 1);
    if (best_cost < 0 || cost < best_cost - 1e-9 || (cost < best_cost + 1e-9 && total < best_total)) {
      best_cost = cost;
      best_total = total;
      best = zc;
    }
  }
  return best;
}

// k and rho*c the same in every phase and independent of T (the products of
// computeStateProperties then select one constant).
static bool props_const(const gm_props* p) {
  return p && p->k_powder == p->k_bulk_a0 && p->k_fluid == p->k_bulk_a0 && p->k_bulk_a1 == 0.0 &&
         p->cp_solid_a1 == 0.0 && p->cp_mushy == p->cp_solid_a0 && p->cp_fluid == p->cp_solid_a0;
}

static int level_flags(const gm_level_args* g, const gm_props* p) {
  int f = 0;
  if (!g->k_arr && props_const(p)) f |= LF_CONST;
  if (g->laser) f |= LF_LASER;
  if (g->rhs_box) f |= LF_BOX;
  if (g->F_full || g->corr_full) f |= LF_FULL;
  if (g->k_arr) f |= LF_KARR;
  if (g->accum) f |= LF_ACCUM;
  if (g->surface) f |= LF_SURF;
  if (g->clamp) f |= LF_CLAMP;
  if (g->inactive_amb) f |= LF_INACT;
  if (g->bc_mode == 1) f |= LF_BC1;
  if (g->bc_mode == 2) f |= LF_BC2;
  if (g->bc_mode == 3) f |= LF_BC3;
  if (g->ph_in) f |= LF_PHIN;
  if (g->ph_out) f |= LF_PHOUT;
  return f;
}

// Launch shapes measured by gm_level_autotune, per (dtype, feature flags,
// grid); gm_level_step uses them when the caller leaves zchunk at 0.
struct TuneKey {
  int dtype, flags, nx, ny, nz;
  bool operator<(const TuneKey& o) const {
    if (dtype != o.dtype) return dtype < o.dtype;
    if (flags != o.flags) return flags < o.flags;
    if (nx != o.nx) return nx < o.nx;
    if (ny != o.ny) return ny < o.ny;
    return nz < o.nz;
  }
};
// A launch shape: kernel 0 = element tiles (tile_x 32 -> 32 x 8, 16 -> 16 x
// 16), kernel 1 = separable stencil (wys thread rows of `rows` y rows each);
// zchunk = node planes per CTA.
struct TuneVal {
  int kernel, tile_x, wys, rows, zchunk;
};
static std::map<TuneKey, TuneVal> g_tuned;
static std::mutex g_tuned_mutex;

static bool tuned_shape(const TuneKey& k, TuneVal* v) {
  std::lock_guard<std::mutex> lock(g_tuned_mutex);
  auto it = g_tuned.find(k);
  if (it == g_tuned.end()) return false;
  *v = it->second;
  return true;
}

template <typename real, int FL, int TXv, int BYv>
static void launch_shape(const LevelK<real>& a, int zc_req, cudaStream_t st) {
  const int gx = cdiv(a.nx, TXv - 1), gy = cdiv(a.ny, BYv - 1);
  int zc = zc_req > 0 ? zc_req : auto_zchunk<real, TXv, BYv, FL>(gx * gy, a.nz);
  if (zc > ZMAX) zc = ZMAX;
  LevelK<real> b = a;
  b.zchunk = zc;
  dim3 grid(gx, gy, cdiv(a.nz, zc)), block(TXv, BYv);
  level_step_kernel<real, TXv, BYv, FL><<<grid, block, 0, st>>>(b);
}

// Element-tile launch: tile_x 16 -> 16 x 16, else 32 x 8; zc_req <= 0: the
// z-chunk model.
template <typename real, int FL>
static void launch_variant(const LevelK<real>& a, int zc_req, cudaStream_t st, int tile_x) {
  if (tile_x == 16)
    launch_shape<real, FL, 16, 16>(a, zc_req, st);
  else
    launch_shape<real, FL, LT_X, LT_Y>(a, zc_req, st);
}

// The separable kernel serves the constant-property Level-1/2/3 variants
// when no node lies above the active element planes (or those nodes are
// reset to T_amb).
static bool sep_eligible(const gm_level_args* g, int fl) {
  if (!(fl & LF_CONST)) return false;
  const int b = fl & ~LF_CONST;
  if (b != LF_L3 && b != LF_L3ACC && b != LF_L2 && b != LF_L1) return false;
  return g->ne_planes == g->nz - 1 || (fl & LF_INACT);
}

// Separable launch: CTAs of `warps` warps (one x-tile, warps x BYT rows),
// v.zchunk <= SEP_ZMAX planes.
template <typename real, int FL, int BYT>
static void launch_sep_t(const LevelK<real>& a, int warps, int zc, bool pdl, cudaStream_t st) {
  LevelK<real> b = a;
  b.zchunk = zc;
  // z-slices: the marching chunks, the top plane, the Dirichlet nodes
  const dim3 grid(cdiv(a.nx, SEP_TILE), cdiv(a.ny, warps * BYT),
                  sep_march_chunks(a.nz, a.ne_planes, (FL & LF_INACT) != 0, zc) + 2);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(32 * warps);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  cudaLaunchKernelEx(&cfg, level_sep_kernel<real, BYT, FL>, b);
}

template <typename real>
static int launch_sep(const LevelK<real>& a, int fl, const TuneVal& v, bool pdl, cudaStream_t st) {
  if ((v.rows != 1 && v.rows != 2 && v.rows != 4) || v.wys < 1 || v.wys > 8 || v.zchunk < 1 ||
      v.zchunk > SEP_ZMAX)
    return GM_ERR_ARG;
  switch (fl) {
#define GM_SEP(V)                                                  \
  case V | LF_CONST:                                               \
    if (v.rows == 1)                                               \
      launch_sep_t<real, V | LF_CONST, 1>(a, v.wys, v.zchunk, pdl, st); \
    else if (v.rows == 2)                                          \
      launch_sep_t<real, V | LF_CONST, 2>(a, v.wys, v.zchunk, pdl, st); \
    else                                                           \
      launch_sep_t<real, V | LF_CONST, 4>(a, v.wys, v.zchunk, pdl, st); \
    break;
    GM_SEP(LF_L3)
    GM_SEP(LF_L3ACC)
    GM_SEP(LF_L2)
    GM_SEP(LF_L1)
#undef GM_SEP
    default:
      return GM_ERR_ARG;
  }
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

// Untuned separable shape: 2 rows a thread, 4-warp CTAs (the best family on
// the 161 x 161 x 41 Level-3 window), and the z-chunk (<= SEP_ZMAX) whose CTA
// count best fills the SMs: busiest SM's CTAs x (planes + 2 halo planes).
template <typename real>
static TuneVal sep_default(const gm_level_args* g, bool inact) {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    sms = n > 0 ? n : 152;
  }
  TuneVal v{1, SEP_TILE, 4, 2, 1};
  const int res = sizeof(real) == 4 ? 6 : 3;  // resident 4-warp CTAs per SM (about 80 / 128+ registers a thread)
  const long long gxy = (long long)cdiv(g->nx, SEP_TILE) * cdiv(g->ny, v.wys * v.rows);
  double best = -1;
  for (int zc = 2; zc <= min(g->nz, SEP_ZMAX); ++zc) {
    const long long ctas = gxy * (sep_march_chunks(g->nz, g->ne_planes, inact, zc) + 1);
    const long long waves = (ctas + (long long)sms * res - 1) / ((long long)sms * res);
    const double cost = (double)waves * (zc + 2);
    if (best < 0 || cost < best - 1e-9) {
      best = cost;
      v.zchunk = zc;
    }
  }
  if (g->nz < 2) v.zchunk = 1;
  return v;
}

template <typename real>
static LevelK<real> make_levelk(const gm_level_args* g, const gm_props* pr) {
  LevelK<real> a;
  a.nx = g->nx;
  a.ny = g->ny;
  a.nz = g->nz;
  a.ne_planes = g->ne_planes;
  a.ox = g->origin[0];
  a.oy = g->origin[1];
  a.oz = g->origin[2];
  a.hx = g->h[0];
  a.hy = g->h[1];
  a.hz = g->h[2];
  a.dt = g->dt;
  a.T_in = (const real*)g->T_in;
  a.T_out = (real*)g->T_out;
  a.ph_in = g->ph_in;
  a.ph_out = g->ph_out;
  a.substrate = g->substrate;
  a.k_arr = (const real*)g->k_arr;
  a.rc_arr = (const real*)g->rc_arr;
  a.F_full = (const real*)g->F_full;
  a.corr_full = (const real*)g->corr_full;
  a.rhs_box = (const real*)g->rhs_box;
  for (int i = 0; i < 6; ++i) a.box[i] = g->box[i];
  a.laser = g->laser;
  a.surface = g->surface;
  a.bc_mode = g->bc_mode;
  a.inactive_amb = g->inactive_amb;
  a.clamp = g->clamp;
  for (int i = 0; i < 5; ++i) a.face[i] = (real)g->face[i];
  a.bc_new = (const real*)g->bc_new;
  a.bc_old = (const real*)g->bc_old;
  a.bc_alpha = (real)g->bc_alpha;
  a.bc_beta = (real)g->bc_beta;
  a.bc_map = make_map3<real>(g->bc_map);
  a.accum = (real*)g->accum;
  a.max_accum = (real*)g->max_accum;
  a.status = g->status;
  a.p = make_props<real>(*pr);
  const double hx = g->h[0], hy = g->h[1], hz = g->h[2];
  for (int m = 0; m < 8; ++m) {
    const int mx = m & 1, my = (m >> 1) & 1, mz = (m >> 2) & 1;
    const double Mx = mx ? hx / 6 : hx / 2, My = my ? hy / 6 : hy / 2, Mz = mz ? hz / 6 : hz / 2;
    const double Kx = mx ? 2 / hx : 0, Ky = my ? 2 / hy : 0, Kz = mz ? 2 / hz : 0;
    a.lam[m] = (real)((Kx * My * Mz + Mx * Ky * Mz + Mx * My * Kz) / 8.0);
  }
  a.wvol = (real)(hx * hy * hz / 8.0);
  a.w2 = (real)(hx * hy / 4.0);
  const double r = pr->laser_radius, d = pr->laser_depth;
  a.inv_r2 = 1.0 / (r * r);
  a.inv_d2 = 1.0 / (d * d);
  const double rc = 1.0 / (r * sqrt(M_PI)), dc = 1.0 / (d * sqrt(M_PI));
  a.src_c = 6.0 * sqrt(3.0) * pr->laser_eta * rc * rc * dc * (hx * hy * hz / 8.0);
  a.zchunk = g->zchunk;
  a.rh[0] = (real)hx;
  a.rh[1] = (real)hy;
  a.rh[2] = (real)hz;
  a.rir2 = (real)a.inv_r2;
  a.rid2 = (real)a.inv_d2;
  const double kc = pr->k_fluid / 1000.0;
  a.sa1 = (real)(kc * hy * hz / (36.0 * hx));
  a.sb1 = (real)(kc * hx * hz / (36.0 * hy));
  a.sb2 = (real)(kc * hx * hy / (36.0 * hz));
  a.smass = (real)(hx * hy * hz * pr->rho * pr->cp_fluid);
  a.src_tab = (const real*)g->src_tab;
  return a;
}

// The feature combination of a call: one of the specialised instantiations,
// or the generic one.
static int variant_of(int flags) {
  const int b = flags & ~LF_CONST;
  return (b == LF_L3 || b == LF_L3ACC || b == LF_L2 || b == LF_L1) ? flags : LF_GENERIC;
}

// One case per specialised variant (with and without constant properties).
#define GM_LEVEL_VARIANTS(X) \
  X(LF_L3)                   \
  X(LF_L3ACC)                \
  X(LF_L2)                   \
  X(LF_L1)                   \
  X(LF_L3 | LF_CONST)        \
  X(LF_L3ACC | LF_CONST)     \
  X(LF_L2 | LF_CONST)        \
  X(LF_L1 | LF_CONST)

// One level step with shape `sh`; sh.kernel < 0: the tuned shape for this
// call if gm_level_autotune measured one (and the caller left zchunk at 0),
// else the separable kernel where eligible, else 32 x 8 element tiles.
template <typename real>
static int launch_level(const gm_level_args* g, const gm_props* pr, cudaStream_t st,
                        TuneVal sh = TuneVal{-1, 0, 0, 0, 0}) {
  const LevelK<real> a = make_levelk<real>(g, pr);
  const int fl = level_flags(g, pr);
  const bool sep_ok = sep_eligible(g, fl);
  if (sh.kernel < 0) {
    TuneVal v;
    if (g->zchunk <= 0 && tuned_shape(TuneKey{g->dtype, fl, g->nx, g->ny, g->nz}, &v)) {
      sh = v;
    } else if (sep_ok) {
      sh = sep_default<real>(g, (fl & LF_INACT) != 0);
      if (g->zchunk > 0) sh.zchunk = g->zchunk;
    } else {
      sh = TuneVal{0, 0, 0, 0, g->zchunk};
    }
  }
  if (sh.kernel == 1) return sep_ok ? launch_sep<real>(a, fl, sh, g->pdl != 0, st) : GM_ERR_ARG;
  switch (variant_of(fl)) {
#define GM_CASE(V)                                        \
  case V:                                                 \
    launch_variant<real, V>(a, sh.zchunk, st, sh.tile_x); \
    break;
    GM_LEVEL_VARIANTS(GM_CASE)
#undef GM_CASE
    default:
      launch_variant<real, LF_GENERIC>(a, sh.zchunk, st, sh.tile_x);
  }
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

// Batched launches: the separable kernel (2 rows x 4 warps) when every
// instance is a constant-property call it serves, else 32 x 8 element tiles.
// The descriptor buffer holds a small header {nb, dtype, variant, total
// blocks, kernel, rows, warps}, the per-instance LevelK array
// and the block prefix first[nb + 1]; a launch reads only device memory, so
// it can be captured in a CUDA graph and replayed.
struct BatchHeader {
  int nb, dtype, variant, blocks, kernel, rows, warps;
};
constexpr int SEP_BATCH_ROWS = 2, SEP_BATCH_WARPS = 4;  // separable batch shape
static size_t batch_tab_offset() { return 256; }
template <typename real>
static size_t batch_first_offset(int nb) {
  return (batch_tab_offset() + sizeof(LevelK<real>) * nb + 255) / 256 * 256;
}

template <typename real>
static int prepare_batched(const gm_level_args* g, int nb, const gm_props* p, void* desc, long long desc_bytes,
                           cudaStream_t st, BatchHeader* hdr) {
  std::vector<LevelK<real>> tabs(nb);
  const int fl = level_flags(&g[0], &p[0]);
  std::vector<int> first(nb + 1);
  first[0] = 0;
  bool sep = true;
  for (int b = 0; b < nb; ++b) sep = sep && level_flags(&g[b], &p[b]) == fl && sep_eligible(&g[b], fl);
  if (sep) {
    const bool inact = (fl & LF_INACT) != 0;
    // separable: one z-chunk for the batch from the wave model over all
    // instances' x/y tiles (6 resident 4-warp CTAs per SM in FP32, 3 in FP64)
    static int sms = 0;
    if (sms == 0) {
      int dev = 0, n = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
      sms = n > 0 ? n : 152;
    }
    const int res = sizeof(real) == 4 ? 6 : 3;
    int nzmax = 2;
    for (int b = 0; b < nb; ++b) nzmax = max(nzmax, g[b].nz);
    int zc_batch = 2;
    double best = -1;
    for (int zc = 2; zc <= min(nzmax, SEP_ZMAX); ++zc) {
      long long ctas = 0;
      for (int b = 0; b < nb; ++b)
        ctas += (long long)cdiv(g[b].nx, SEP_TILE) * cdiv(g[b].ny, SEP_BATCH_WARPS * SEP_BATCH_ROWS) *
                (sep_march_chunks(g[b].nz, g[b].ne_planes, inact, zc) + 2);
      const long long waves = (ctas + (long long)sms * res - 1) / ((long long)sms * res);
      const double cost = (double)waves * (zc + 2);
      if (best < 0 || cost < best - 1e-9) {
        best = cost;
        zc_batch = zc;
      }
    }
    for (int b = 0; b < nb; ++b) {
      LevelK<real>& a = tabs[b];
      a = make_levelk<real>(&g[b], &p[b]);
      a.zchunk = (g[b].zchunk > 0 && g[b].zchunk <= SEP_ZMAX) ? g[b].zchunk : zc_batch;
      const long long blocks = (long long)cdiv(a.nx, SEP_TILE) * cdiv(a.ny, SEP_BATCH_WARPS * SEP_BATCH_ROWS) *
                               (sep_march_chunks(a.nz, a.ne_planes, inact, a.zchunk) + 2);
      if (first[b] + blocks >= (1LL << 31)) return GM_ERR_TOO_LARGE;
      first[b + 1] = first[b] + (int)blocks;
    }
    const size_t off = batch_first_offset<real>(nb);
    if ((long long)(off + sizeof(int) * (nb + 1)) > desc_bytes) return GM_ERR_TOO_LARGE;
    *hdr = BatchHeader{nb, g[0].dtype, fl, first[nb], 1, SEP_BATCH_ROWS, SEP_BATCH_WARPS};
    if (cudaMemcpyAsync(desc, hdr, sizeof(BatchHeader), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync((char*)desc + batch_tab_offset(), tabs.data(), sizeof(LevelK<real>) * nb,
                        cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync((char*)desc + off, first.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice, st) !=
            cudaSuccess)
      return GM_ERR_CUDA;
    return GM_OK;
  }
  // one z-chunk for the whole batch: the cost model over all instances'
  // tiles together (a lone small window would be split much finer)
  long long tiles = 0;
  int nzmax = 1;
  for (int b = 0; b < nb; ++b) {
    tiles += (long long)cdiv(g[b].nx, LT_X - 1) * cdiv(g[b].ny, LT_Y - 1);
    nzmax = max(nzmax, g[b].nz);
  }
  const int zc_batch =
      auto_zchunk<real, LT_X, LT_Y, LF_GENERIC>((int)min(tiles, (long long)(1 << 30)), nzmax);
  for (int b = 0; b < nb; ++b) {
    if (level_flags(&g[b], &p[b]) != fl) return GM_ERR_ARG;
    LevelK<real>& a = tabs[b];
    a = make_levelk<real>(&g[b], &p[b]);
    if (a.zchunk <= 0) a.zchunk = zc_batch;
    if (a.zchunk > ZMAX) a.zchunk = ZMAX;
    const long long blocks = (long long)cdiv(a.nx, LT_X - 1) * cdiv(a.ny, LT_Y - 1) * cdiv(a.nz, a.zchunk);
    if (first[b] + blocks >= (1LL << 31)) return GM_ERR_TOO_LARGE;
    first[b + 1] = first[b] + (int)blocks;
  }
  const size_t off = batch_first_offset<real>(nb);
  if ((long long)(off + sizeof(int) * (nb + 1)) > desc_bytes) return GM_ERR_TOO_LARGE;
  *hdr = BatchHeader{nb, g[0].dtype, variant_of(fl), first[nb], 0, 0, 0};
  // pageable sources: each copy returns once the host data has been consumed
  if (cudaMemcpyAsync(desc, hdr, sizeof(BatchHeader), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync((char*)desc + batch_tab_offset(), tabs.data(), sizeof(LevelK<real>) * nb,
                      cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync((char*)desc + off, first.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice, st) !=
          cudaSuccess)
    return GM_ERR_CUDA;
  return GM_OK;
}

template <typename real>
static int launch_batched(const BatchHeader& h, const void* desc, cudaStream_t st) {
  const LevelK<real>* tab = (const LevelK<real>*)((const char*)desc + batch_tab_offset());
  const int* first = (const int*)((const char*)desc + batch_first_offset<real>(h.nb));
  if (h.kernel == 1) {
    if (h.rows != SEP_BATCH_ROWS || h.warps != SEP_BATCH_WARPS) return GM_ERR_ARG;
    const dim3 sblk(32 * SEP_BATCH_WARPS);
    switch (h.variant) {
#define GM_SEPB(V)                                                                                    \
  case V | LF_CONST:                                                                                  \
    level_sep_batched_kernel<real, SEP_BATCH_ROWS, V | LF_CONST><<<h.blocks, sblk, 0, st>>>(tab, first, h.nb); \
    break;
      GM_SEPB(LF_L3)
      GM_SEPB(LF_L3ACC)
      GM_SEPB(LF_L2)
      GM_SEPB(LF_L1)
#undef GM_SEPB
      default:
        return GM_ERR_ARG;
    }
    return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
  }
  const dim3 blk(LT_X, LT_Y);
  switch (h.variant) {
#define GM_CASE(V)                                                                              \
  case V:                                                                                       \
    level_step_batched_kernel<real, LT_X, LT_Y, V><<<h.blocks, blk, 0, st>>>(tab, first, h.nb); \
    break;
    GM_LEVEL_VARIANTS(GM_CASE)
#undef GM_CASE
    default:
      level_step_batched_kernel<real, LT_X, LT_Y, LF_GENERIC><<<h.blocks, blk, 0, st>>>(tab, first, h.nb);
  }
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

static int check_level_args(const gm_level_args* a) {
  if (!a || !a->T_in || !a->T_out || !a->dt || a->T_in == a->T_out) return GM_ERR_ARG;
  if (a->nx < 2 || a->ny < 2 || a->nz < 2 || a->ne_planes < 0 || a->ne_planes > a->nz - 1) return GM_ERR_ARG;
  if ((long long)a->nx * a->ny * a->nz >= (1LL << 31)) return GM_ERR_TOO_LARGE;  // node ids are 32-bit
  if ((a->k_arr == nullptr) != (a->rc_arr == nullptr)) return GM_ERR_ARG;
  if (a->bc_mode == 2 && (!a->bc_new || !a->bc_old || !a->bc_map.elem[0] || !a->bc_map.w[0])) return GM_ERR_ARG;
  if (a->bc_mode == 3 && (!a->bc_new || !a->bc_old)) return GM_ERR_ARG;
  if (a->bc_mode < 0 || a->bc_mode > 3) return GM_ERR_ARG;
  if ((a->accum == nullptr) != (a->max_accum == nullptr)) return GM_ERR_ARG;
  if (a->dtype != GM_F32 && a->dtype != GM_F64) return GM_ERR_ARG;
  return GM_OK;
}

}  // namespace gm

extern "C" int gm_level_step(const gm_level_args* a, const gm_props* p, void* stream) {
  if (!p) return GM_ERR_ARG;
  const int rc = gm::check_level_args(a);
  if (rc != GM_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (a->dtype == GM_F32) return gm::launch_level<float>(a, p, st);
  return gm::launch_level<double>(a, p, st);
}

extern "C" long long gm_level_batched_desc_size(int nb, int dtype) {
  if (nb < 1) return -1;
  const size_t off = dtype == GM_F64 ? gm::batch_first_offset<double>(nb) : gm::batch_first_offset<float>(nb);
  return (long long)(off + sizeof(int) * (nb + 1));
}

extern "C" int gm_level_batched_prepare(const gm_level_args* a, int nb, const gm_props* p, void* desc,
                                        long long desc_bytes, gm_batch_info* info, void* stream) {
  if (!a || !p || !desc || nb < 1 || !info) return GM_ERR_ARG;
  for (int b = 0; b < nb; ++b) {
    const int rc = gm::check_level_args(&a[b]);
    if (rc != GM_OK) return rc;
    if (a[b].dtype != a[0].dtype) return GM_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  gm::BatchHeader h;
  const int rc = a[0].dtype == GM_F32 ? gm::prepare_batched<float>(a, nb, p, desc, desc_bytes, st, &h)
                                      : gm::prepare_batched<double>(a, nb, p, desc, desc_bytes, st, &h);
  if (rc != GM_OK) return rc;
  info->nb = h.nb;
  info->dtype = h.dtype;
  info->variant = h.variant;
  info->blocks = h.blocks;
  info->kernel = h.kernel;
  info->rows = h.rows;
  info->warps = h.warps;
  return GM_OK;
}

extern "C" int gm_level_batched_launch(const void* desc, const gm_batch_info* info, void* stream) {
  if (!desc || !info || info->nb < 1 || info->blocks < 1) return GM_ERR_ARG;
  const gm::BatchHeader h{info->nb, info->dtype, info->variant, info->blocks, info->kernel, info->rows, info->warps};
  cudaStream_t st = (cudaStream_t)stream;
  if (h.dtype == GM_F32) return gm::launch_batched<float>(h, desc, st);
  if (h.dtype == GM_F64) return gm::launch_batched<double>(h, desc, st);
  return GM_ERR_ARG;
}

extern "C" int gm_level_step_batched(const gm_level_args* a, int nb, const gm_props* p, void* desc,
                                     long long desc_bytes, void* stream) {
  gm_batch_info info;
  const int rc = gm_level_batched_prepare(a, nb, p, desc, desc_bytes, &info, stream);
  if (rc != GM_OK) return rc;
  return gm_level_batched_launch(desc, &info, stream);
}

extern "C" int gm_level_step_shape(const gm_level_args* a, const gm_props* p, const gm_level_shape* shape,
                                   void* stream) {
  if (!p || !shape) return GM_ERR_ARG;
  const int rc = gm::check_level_args(a);
  if (rc != GM_OK) return rc;
  if (shape->kernel != 0 && shape->kernel != 1) return GM_ERR_ARG;
  if (shape->kernel == 0 && shape->tile_x != 32 && shape->tile_x != 16) return GM_ERR_ARG;
  const gm::TuneVal v{shape->kernel, shape->tile_x, shape->tile_y, shape->rows, shape->zchunk};
  cudaStream_t st = (cudaStream_t)stream;
  if (a->dtype == GM_F32) return gm::launch_level<float>(a, p, st, v);
  return gm::launch_level<double>(a, p, st, v);
}

namespace gm {

// Times each candidate shape as a CUDA graph of R back-to-back launches of
// `launch(v)` (programmatic dependents of one another, as gm_subcycle issues
// level steps), so that neither host launch overhead nor the launch gaps of
// stream order enter the comparison; on a stream that cannot be captured (the
// legacy default stream) the launches are timed as issued.  One untimed launch
// precedes each candidate.  Returns the fastest in *best / *best_us.
template <typename Launch>
static int time_shapes(const std::vector<TuneVal>& cand, int R, cudaStream_t st, Launch launch, TuneVal* best,
                       float* best_us) {
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return GM_ERR_CUDA;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return GM_ERR_CUDA;
  }
  *best_us = -1.f;
  int status = GM_OK;
  for (const TuneVal& v : cand) {
    status = launch(v);  // untimed first launch
    if (status != GM_OK) break;
    cudaGraphExec_t exec = nullptr;
    if (st && cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      for (int r = 0; r < R && status == GM_OK; ++r) status = launch(v);
      cudaGraph_t graph = nullptr;
      const cudaError_t ec = cudaStreamEndCapture(st, &graph);
      if (status == GM_OK && ec == cudaSuccess && graph &&
          cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess && cudaGraphLaunch(exec, st) == cudaSuccess) {
        cudaEventRecord(e0, st);
        cudaGraphLaunch(exec, st);
        cudaEventRecord(e1, st);
      } else {
        status = status != GM_OK ? status : GM_ERR_CUDA;
      }
      if (graph) cudaGraphDestroy(graph);
    } else {
      cudaGetLastError();  // not capturable: time the launches as issued
      cudaEventRecord(e0, st);
      for (int r = 0; r < R && status == GM_OK; ++r) status = launch(v);
      cudaEventRecord(e1, st);
    }
    if (status != GM_OK) {
      if (exec) cudaGraphExecDestroy(exec);
      break;
    }
    const bool synced = cudaEventSynchronize(e1) == cudaSuccess;
    if (exec) cudaGraphExecDestroy(exec);
    if (!synced) {
      status = GM_ERR_CUDA;
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const float us = 1000.f * ms / R;
    if (*best_us < 0 || us < *best_us) {
      *best_us = us;
      *best = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return status;
}

}  // namespace gm

extern "C" int gm_level_autotune(const gm_level_args* a, const gm_props* p, int reps, gm_tune_result* out,
                                 void* stream) {
  if (!p || reps < 1) return GM_ERR_ARG;
  const int rc = gm::check_level_args(a);
  if (rc != GM_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  // candidates: element tiles 32 x 8 and 16 x 16, and (where eligible) the
  // separable kernel with 2 or 4 rows a thread and 1, 2 or 4 thread rows,
  // each over the distinct z-chunks of 2..64 planes
  std::vector<gm::TuneVal> cand;
  std::vector<int> zcs;
  for (int nch = gm::cdiv(a->nz, gm::ZMAX), last = -1; nch <= a->nz; ++nch) {
    const int zc = gm::cdiv(a->nz, nch);
    if (zc == last || zc < 2) continue;
    last = zc;
    zcs.push_back(zc);
  }
  for (int tx : {gm::LT_X, 16})
    for (int zc : zcs) cand.push_back(gm::TuneVal{0, tx, 0, 0, zc});
  if (gm::sep_eligible(a, gm::level_flags(a, p)))
    for (int rows : {1, 2, 4})
      for (int warps : {2, 4, 8})
        for (int zc : zcs)
          if (zc <= gm::SEP_ZMAX) cand.push_back(gm::TuneVal{1, gm::SEP_TILE, warps, rows, zc});
  gm_level_args b = *a;
  b.pdl = 1;  // the timed launches read the same dt, laser and factors throughout
  auto launch = [&](const gm::TuneVal& v) {
    return b.dtype == GM_F32 ? gm::launch_level<float>(&b, p, st, v) : gm::launch_level<double>(&b, p, st, v);
  };
  gm::TuneVal best{0, gm::LT_X, 0, 0, 0};
  float best_us = -1.f;
  const int status = gm::time_shapes(cand, 4 * reps, st, launch, &best, &best_us);
  if (status != GM_OK) return status;
  {
    std::lock_guard<std::mutex> lock(gm::g_tuned_mutex);
    gm::g_tuned[gm::TuneKey{a->dtype, gm::level_flags(a, p), a->nx, a->ny, a->nz}] = best;
  }
  if (out) {
    out->kernel = best.kernel;
    out->zchunk = best.zchunk;
    out->us = best_us;
    if (best.kernel == 1) {
      out->tile_x = gm::SEP_TILE;
      out->tile_y = best.wys;
      out->rows = best.rows;
    } else {
      out->tile_x = best.tile_x;
      out->tile_y = best.tile_x == 16 ? 16 : gm::LT_Y;
      out->rows = 1;
    }
  }
  return GM_OK;
}

// ---------------------------------------------------------------------------
// The N3 Level-3 steps of one Level-2 step in one cooperative launch, each
// step the separable one-step kernel's body over its tiles (so results are
// the one-step kernel's, bit for bit), the fields in L2 between steps, a grid
// barrier between steps.  It removes the launch ramp and drain of N3 - 1
// launches; the barrier costs one L2 round trip per CTA and step.
// ---------------------------------------------------------------------------
namespace gm {

struct StepsK {
  int nsteps, nsub, tiles, gx, gy;
  const double* rows;
  const void* src_tab;
  int src_stride;
  const void* T_in;
  void* T_out;
  void* tb0;
  void* tb1;
  const uint8_t* ph_in;
  uint8_t* ph_out;
  unsigned* counter;
  unsigned base;
  int* status;
};

constexpr long long STEPS_WAIT_CYCLES = 2000000000LL;

template <typename real, int BYT, int FL>
__global__ void __launch_bounds__(256, sep_min_blocks<real, BYT>()) level_sep_steps_kernel(const LevelK<real> a0, const StepsK k) {
  __shared__ LevelK<real> a;
  __shared__ int s_abort;
  if (threadIdx.x == 0) {
    a = a0;
    s_abort = 0;
  }
  const int gz = k.tiles / (k.gx * k.gy);
  for (int s = 0; s < k.nsteps; ++s) {
    __syncthreads();
    if (threadIdx.x == 0) {  // this step's inputs and outputs
      a.T_in = (const real*)(s == 0 ? k.T_in : ((s & 1) ? k.tb0 : k.tb1));
      a.T_out = (real*)(s == k.nsteps - 1 ? k.T_out : ((s & 1) ? k.tb1 : k.tb0));
      a.ph_in = s == 0 ? k.ph_in : k.ph_out;  // a node's phase is read and written by its own thread only
      a.ph_out = k.ph_out;
      a.dt = k.rows + 7LL * s + 5;
      a.laser = k.rows + 7LL * s;
      a.src_tab = (const real*)k.src_tab + (long long)s * k.src_stride;
      const double al = (double)(s + 1) / (double)k.nsub;
      a.bc_alpha = (real)al;
      a.bc_beta = (real)(1.0 - al);
    }
    __syncthreads();
    for (int t = blockIdx.x; t < k.tiles; t += gridDim.x) {
      const int bx = t % k.gx, by = (t / k.gx) % k.gy, bz = t / (k.gx * k.gy);
      sep_body<real, BYT, FL>(a, bx, by, bz, k.gx, k.gy, gz - 1);
    }
    if (s == k.nsteps - 1) break;
    // grid barrier: every tile of step s is written before any CTA reads it
    __syncthreads();
    if (threadIdx.x == 0) {
      const unsigned target = k.base + (unsigned)((s + 1) * gridDim.x);
      asm volatile("fence.acq_rel.gpu;\n red.relaxed.gpu.global.add.u32 [%0], 1;" ::"l"(k.counter) : "memory");
      const long long t0 = clock64();
      unsigned v;
      for (;;) {
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(k.counter) : "memory");
        if ((int)(v - target) >= 0) break;
        if (clock64() - t0 > STEPS_WAIT_CYCLES) {
          s_abort = 1;
          atomicOr(k.status, GM_PERSIST_TIMEOUT);
          break;
        }
      }
    }
    __syncthreads();
    if (s_abort) return;
  }
}

template <typename real, int BYT, int FL>
static int launch_steps_t(const LevelK<real>& a, StepsK k, int warps, cudaStream_t st) {
  auto kern = level_sep_steps_kernel<real, BYT, FL>;
  static int sms = 0;
  if (sms == 0) {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    sms = n > 0 ? n : 152;
  }
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 32 * warps, 0) != cudaSuccess || occ < 1) {
    cudaGetLastError();
    return GM_ERR_UNSUPPORTED;
  }
  const int grid = k.tiles < occ * sms ? k.tiles : occ * sms;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(32 * warps);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;  // every CTA resident: the grid barrier cannot starve
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, a, k) == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

template <typename real>
static int launch_steps(const gm_steps_args* g, const gm_props* pr, cudaStream_t st) {
  const gm_level_args* la = &g->level;
  const int fl = level_flags(la, pr);
  if (!sep_eligible(la, fl) || (fl != (LF_L3 | LF_CONST) && fl != (LF_L3ACC | LF_CONST))) return GM_ERR_UNSUPPORTED;
  TuneVal v;
  if (la->zchunk > 0 || !tuned_shape(TuneKey{la->dtype, fl, la->nx, la->ny, la->nz}, &v) || v.kernel != 1)
    v = sep_default<real>(la, false);
  if (la->zchunk > 0) v.zchunk = la->zchunk;
  if ((v.rows != 1 && v.rows != 2 && v.rows != 4) || v.wys < 1 || v.wys > 8 || v.zchunk < 1 || v.zchunk > SEP_ZMAX)
    return GM_ERR_ARG;
  LevelK<real> a = make_levelk<real>(la, pr);
  a.zchunk = v.zchunk;
  StepsK k;
  k.nsteps = g->nsteps;
  k.nsub = g->nsub;
  k.gx = cdiv(la->nx, SEP_TILE);
  k.gy = cdiv(la->ny, v.wys * v.rows);
  const long long tiles =
      (long long)k.gx * k.gy * (sep_march_chunks(la->nz, la->ne_planes, false, v.zchunk) + 2);
  if (tiles >= (1LL << 31)) return GM_ERR_TOO_LARGE;
  k.tiles = (int)tiles;
  k.rows = g->rows;
  k.src_tab = g->src_tab;
  k.src_stride = la->nx + la->ny + la->nz;
  k.T_in = la->T_in;
  k.T_out = la->T_out;
  k.tb0 = g->tbuf[0];
  k.tb1 = g->tbuf[1];
  k.ph_in = la->ph_in;
  k.ph_out = la->ph_out;
  k.counter = g->counter;
  k.base = g->base;
  k.status = g->status;
  const int fa = LF_L3 | LF_CONST, fb = LF_L3ACC | LF_CONST;
  if (v.rows == 1)
    return fl == fa ? launch_steps_t<real, 1, fa>(a, k, v.wys, st) : launch_steps_t<real, 1, fb>(a, k, v.wys, st);
  if (v.rows == 2)
    return fl == fa ? launch_steps_t<real, 2, fa>(a, k, v.wys, st) : launch_steps_t<real, 2, fb>(a, k, v.wys, st);
  return fl == fa ? launch_steps_t<real, 4, fa>(a, k, v.wys, st) : launch_steps_t<real, 4, fb>(a, k, v.wys, st);
}

}  // namespace gm

extern "C" int gm_level3_steps(const gm_steps_args* g, const gm_props* p, void* stream) {
  if (!g || !p || g->nsteps < 1 || g->nsub < 1 || !g->rows || !g->src_tab || !g->tbuf[0] || !g->tbuf[1] ||
      !g->counter || !g->status)
    return GM_ERR_ARG;
  const gm_level_args* la = &g->level;
  const int rc = gm::check_level_args(la);
  if (rc != GM_OK) return rc;
  if (!la->ph_in || !la->ph_out || la->bc_mode != 3 || !la->laser) return GM_ERR_ARG;
  const void* bufs[4] = {la->T_in, la->T_out, g->tbuf[0], g->tbuf[1]};
  for (int i = 0; i < 4; ++i)
    for (int j = i + 1; j < 4; ++j)
      if (bufs[i] == bufs[j]) return GM_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (la->dtype == GM_F32) return gm::launch_steps<float>(g, p, st);
  return gm::launch_steps<double>(g, p, st);
}

// ---------------------------------------------------------------------------
// Two Level-3 fine steps in one launch (gm_sep2.cuh).
// ---------------------------------------------------------------------------
#include "gm_sep2.cuh"

namespace gm {

constexpr int LF_TWO = 1 << 14;  // tune-key bit: the two-step kernel's shape

template <typename real, int FL, int BYT>
static void launch_sep2_t(const LevelK<real>& a, const Step2<real>& b, int warps, int zc, bool pdl, cudaStream_t st) {
  LevelK<real> c = a;
  c.zchunk = zc;
  // z-slices: the marching chunks, the two top planes, the Dirichlet nodes
  const dim3 grid(cdiv(a.nx, SEP2_TILE), cdiv(a.ny, warps * BYT), sep2_march_chunks(a.ne_planes, zc) + 2);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(32 * warps);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  cudaLaunchKernelEx(&cfg, level_sep2_kernel<real, BYT, FL>, c, b);
}

// The two-step kernel serves constant-property Level-3 calls (laser factors
// from tables for both steps, surface flux, clamp, ring arrays, phase in and
// out, optional melt time) whose nodes are all at or below the top plane.
static bool sep2_eligible(const gm_level2_args* g, int fl) {
  const gm_level_args& a = g->level;
  return (fl == (LF_L3 | LF_CONST) || fl == (LF_L3ACC | LF_CONST)) && a.ne_planes == a.nz - 1 && a.nz >= 3 &&
         a.src_tab && g->src_tab2 && g->dt2;
}

template <typename real>
static int launch_sep2(const gm_level2_args* g, const gm_props* pr, const TuneVal& v, cudaStream_t st) {
  const gm_level_args* la = &g->level;
  const int fl = level_flags(la, pr);
  if (!sep2_eligible(g, fl)) return GM_ERR_UNSUPPORTED;
  if ((v.rows != 1 && v.rows != 2 && v.rows != 4) || v.wys < 1 || v.wys > 8 || v.zchunk < 1 ||
      v.zchunk > SEP2_ZMAX)
    return GM_ERR_ARG;
  const LevelK<real> a = make_levelk<real>(la, pr);
  Step2<real> b;
  b.dt = g->dt2;
  b.src_tab = (const real*)g->src_tab2;
  b.bc_alpha = (real)g->bc_alpha2;
  b.bc_beta = (real)g->bc_beta2;
  const bool pdl = la->pdl != 0;
  constexpr int fa = LF_L3 | LF_CONST, fb = LF_L3ACC | LF_CONST;
  if (v.rows == 1) {
    if (fl == fa)
      launch_sep2_t<real, fa, 1>(a, b, v.wys, v.zchunk, pdl, st);
    else
      launch_sep2_t<real, fb, 1>(a, b, v.wys, v.zchunk, pdl, st);
  } else if (v.rows == 2) {
    if (fl == fa)
      launch_sep2_t<real, fa, 2>(a, b, v.wys, v.zchunk, pdl, st);
    else
      launch_sep2_t<real, fb, 2>(a, b, v.wys, v.zchunk, pdl, st);
  } else {
    if (fl == fa)
      launch_sep2_t<real, fa, 4>(a, b, v.wys, v.zchunk, pdl, st);
    else
      launch_sep2_t<real, fb, 4>(a, b, v.wys, v.zchunk, pdl, st);
  }
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

// Untuned two-step shape: 2 rows a thread, 4-warp CTAs, and the z-chunk whose
// CTA count best fills the SMs (busiest SM's CTAs x (planes + 4 halo planes)).
static TuneVal sep2_default(const gm_level_args* g) {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    sms = n > 0 ? n : 152;
  }
  TuneVal v{2, SEP2_TILE, 4, 2, 1};
  const int res = g->dtype == GM_F32 ? 4 : 2;  // resident 4-warp CTAs per SM
  const long long gxy = (long long)cdiv(g->nx, SEP2_TILE) * cdiv(g->ny, v.wys * v.rows);
  const int nplanes = g->ne_planes - 2;
  double best = -1;
  for (int zc = 1; zc <= min(max(nplanes, 1), SEP2_ZMAX); ++zc) {
    const long long ctas = gxy * (sep2_march_chunks(g->ne_planes, zc) + 1);
    const long long waves = (ctas + (long long)sms * res - 1) / ((long long)sms * res);
    const double cost = (double)waves * (zc + 4);
    if (best < 0 || cost < best - 1e-9) {
      best = cost;
      v.zchunk = zc;
    }
  }
  return v;
}

static int check_level2_args(const gm_level2_args* g, const gm_props* p) {
  if (!g || !p) return GM_ERR_ARG;
  const int rc = check_level_args(&g->level);
  if (rc != GM_OK) return rc;
  const gm_level_args& a = g->level;
  if (!g->dt2 || !a.ph_in || !a.ph_out || a.ph_in == a.ph_out || a.bc_mode != 3 || !a.laser) return GM_ERR_ARG;
  if (!sep2_eligible(g, level_flags(&a, p))) return GM_ERR_UNSUPPORTED;
  return GM_OK;
}

template <typename real>
static int launch_level2(const gm_level2_args* g, const gm_props* p, cudaStream_t st, TuneVal sh) {
  if (sh.kernel < 0) {
    const gm_level_args* la = &g->level;
    TuneVal v;
    if (la->zchunk <= 0 && tuned_shape(TuneKey{la->dtype, level_flags(la, p) | LF_TWO, la->nx, la->ny, la->nz}, &v))
      sh = v;
    else
      sh = sep2_default(la);
    if (la->zchunk > 0) sh.zchunk = la->zchunk;
  }
  return launch_sep2<real>(g, p, sh, st);
}

}  // namespace gm

extern "C" int gm_level_step2(const gm_level2_args* a, const gm_props* p, void* stream) {
  const int rc = gm::check_level2_args(a, p);
  if (rc != GM_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const gm::TuneVal none{-1, 0, 0, 0, 0};
  if (a->level.dtype == GM_F32) return gm::launch_level2<float>(a, p, st, none);
  return gm::launch_level2<double>(a, p, st, none);
}

extern "C" int gm_level_step2_shape(const gm_level2_args* a, const gm_props* p, const gm_level_shape* shape,
                                    void* stream) {
  if (!shape) return GM_ERR_ARG;
  const int rc = gm::check_level2_args(a, p);
  if (rc != GM_OK) return rc;
  if (shape->kernel != 2) return GM_ERR_ARG;
  const gm::TuneVal v{2, gm::SEP2_TILE, shape->tile_y, shape->rows, shape->zchunk};
  cudaStream_t st = (cudaStream_t)stream;
  if (a->level.dtype == GM_F32) return gm::launch_level2<float>(a, p, st, v);
  return gm::launch_level2<double>(a, p, st, v);
}

extern "C" int gm_level_autotune2(const gm_level2_args* a, const gm_props* p, int reps, gm_tune_result* out,
                                  void* stream) {
  if (reps < 1) return GM_ERR_ARG;
  const int rc = gm::check_level2_args(a, p);
  if (rc != GM_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int nplanes = a->level.ne_planes - 2;
  std::vector<int> zcs;
  for (int nch = gm::cdiv(nplanes > 0 ? nplanes : 1, gm::SEP2_ZMAX), last = -1; nch <= (nplanes > 0 ? nplanes : 1);
       ++nch) {
    const int zc = gm::cdiv(nplanes > 0 ? nplanes : 1, nch);
    if (zc == last) continue;
    last = zc;
    zcs.push_back(zc);
  }
  std::vector<gm::TuneVal> cand;
  for (int rows : {1, 2, 4})
    for (int warps : {2, 4, 8})
      for (int zc : zcs) cand.push_back(gm::TuneVal{2, gm::SEP2_TILE, warps, rows, zc});
  gm_level2_args b = *a;
  b.level.pdl = 1;
  auto launch = [&](const gm::TuneVal& v) {
    return b.level.dtype == GM_F32 ? gm::launch_level2<float>(&b, p, st, v) : gm::launch_level2<double>(&b, p, st, v);
  };
  gm::TuneVal best{2, gm::SEP2_TILE, 4, 2, 1};
  float best_us = -1.f;
  const int status = gm::time_shapes(cand, 4 * reps, st, launch, &best, &best_us);
  if (status != GM_OK) return status;
  {
    std::lock_guard<std::mutex> lock(gm::g_tuned_mutex);
    gm::g_tuned[gm::TuneKey{a->level.dtype, gm::level_flags(&a->level, p) | gm::LF_TWO, a->level.nx, a->level.ny,
                            a->level.nz}] = best;
  }
  if (out) {
    out->kernel = 2;
    out->zchunk = best.zchunk;
    out->us = best_us;
    out->tile_x = gm::SEP2_TILE;
    out->tile_y = best.wys;
    out->rows = best.rows;
  }
  return GM_OK;
}

extern "C" const char* gm_version(void) { return "gomelt-gb300 0.1 (sm_103a)"; }

// ---------------------------------------------------------------------------
// Stand-alone pieces of the level step (the reference's separate functions).
// ---------------------------------------------------------------------------
namespace gm {

// computeStateProperties (:2567-2614): new phase byte, optional k and rho*c.
template <typename real>
__global__ void state_props_kernel(long long n, const real* T, const uint8_t* ph_in, uint8_t* ph_out, real* k_out,
                                   real* rc_out, long long substrate, const Props<real> p) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    real k, c;
    const uint8_t ph = node_props(p, T[i], ph_in ? ph_in[i] : (uint8_t)0, i < substrate, k, c);
    if (ph_out) ph_out[i] = ph;
    if (k_out) k_out[i] = k;
    if (rc_out) rc_out[i] = c;
  }
}

// computeSourcesL3 (:2960-3012): F[node] += c P Sx[ix] Sy[iy] Sz[iz].
template <typename real>
__global__ void fine_source_kernel(int nx, int ny, int nz, double ox, double oy, double oz, double hx, double hy,
                                   double hz, const double* laser, double rsq, double dsq, double src_c, real* F) {
  const long long n = (long long)nx * ny * nz;
  const double vx = laser[0], vy = laser[1], vz = laser[2];
  const double c = src_c * laser[6];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int ix = (int)(i % nx), iy = (int)((i / nx) % ny), iz = (int)(i / ((long long)nx * ny));
    F[i] += (real)(c * src_factor<double>(ix, nx, ox - vx, hx, 1.0 / rsq) *
                   src_factor<double>(iy, ny, oy - vy, hy, 1.0 / rsq) * src_factor<double>(iz, nz, oz - vz, hz, 1.0 / dsq));
  }
}

// Laser factors of many fine steps on one window, as the separable level
// step uses them (the same expressions, so the step's results do not change):
// row i of tab = [nx] P c Sx[ix], [ny] Sy[iy], [nz] Sz[iz] for laser row i.
template <typename real>
__global__ void fine_source_tables_kernel(int nx, int ny, int nz, double ox, double oy, double oz, real hx, real hy,
                                          real hz, const double* rows, int nrows, real ir2, real id2, double src_c,
                                          real* tab) {
  const int L = nx + ny + nz;
  const long long n = (long long)nrows * L;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t / L), j = (int)(t - (long long)i * L);
    const double* laser = rows + 7LL * i;
    real v;
    if (j < nx) {
      const real rx = (real)(ox - laser[0]), srcP = (real)(src_c * laser[6]);
      v = rmul(srcP, src_factor<real>(j, nx, rx, hx, ir2));
    } else if (j < nx + ny) {
      v = src_factor<real>(j - nx, ny, (real)(oy - laser[1]), hy, ir2);
    } else {
      v = src_factor<real>(j - nx - ny, nz, (real)(oz - laser[2]), hz, id2);
    }
    tab[t] = v;
  }
}

// computeConvRadBC (:2207-2301): flux of the top faces of element plane
// ne_planes-1 into the nodes of plane ne_planes; one thread per node gathers
// its (up to four) faces.
template <typename real>
__global__ void surface_kernel(int nx, int ny, int kt, double hx, double hy, const real* T, real* F, const Props<real> p) {
  const real PQ = (real)0.78867513459481288225, MQ = (real)0.21132486540518711775;
  const long long nxy = (long long)nx * ny;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nxy; i += (long long)gridDim.x * blockDim.x) {
    const int ix = (int)(i % nx), iy = (int)(i / nx);
    const real w2 = (real)(hx * hy / 4.0);
    real acc = 0;
    for (int fy = iy - 1; fy <= iy; ++fy) {
      if (fy < 0 || fy >= ny - 1) continue;
      for (int fx = ix - 1; fx <= ix; ++fx) {
        if (fx < 0 || fx >= nx - 1) continue;
        const long long b = fx + (long long)fy * nx + (long long)kt * nxy;
        const real t00 = T[b], t10 = T[b + 1], t01 = T[b + nx], t11 = T[b + nx + 1];
        const int ax = ix - fx, ay = iy - fy;
        for (int qy = 0; qy < 2; ++qy)
          for (int qx = 0; qx < 2; ++qx) {
            const real px0 = qx ? MQ : PQ, px1 = qx ? PQ : MQ, py0 = qy ? MQ : PQ, py1 = qy ? PQ : MQ;
            const real Tq = px0 * py0 * t00 + px1 * py0 * t10 + px0 * py1 * t01 + px1 * py1 * t11;
            const real q = surface_flux(p, Tq) * w2;
            acc += (ax ? px1 : px0) * (ay ? py1 : py0) * q;
          }
      }
    }
    F[i + (long long)kt * nxy] += acc;
  }
}

inline int lgrid(long long n) {
  long long g = (n + 255) / 256;
  if (g > 152 * 32) g = 152 * 32;
  return g < 1 ? 1 : (int)g;
}

}  // namespace gm

extern "C" int gm_state_properties(const gm_state_props_args* a, const gm_props* p, void* stream) {
  if (!a || !p || !a->T || a->n < 0 || a->ph_in == a->ph_out) return GM_ERR_ARG;
  if ((a->k_out == nullptr) != (a->rc_out == nullptr)) return GM_ERR_ARG;
  if (a->n == 0) return GM_OK;
  cudaStream_t st = (cudaStream_t)stream;
  if (a->dtype == GM_F32)
    gm::state_props_kernel<float><<<gm::lgrid(a->n), 256, 0, st>>>(a->n, (const float*)a->T, a->ph_in, a->ph_out,
                                                                    (float*)a->k_out, (float*)a->rc_out, a->substrate,
                                                                    gm::make_props<float>(*p));
  else if (a->dtype == GM_F64)
    gm::state_props_kernel<double><<<gm::lgrid(a->n), 256, 0, st>>>(a->n, (const double*)a->T, a->ph_in, a->ph_out,
                                                                     (double*)a->k_out, (double*)a->rc_out,
                                                                     a->substrate, gm::make_props<double>(*p));
  else
    return GM_ERR_ARG;
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_fine_source(int dtype, const int nodes[3], const double origin[3], const double h[3],
                              const double* laser, const gm_props* p, void* F, void* stream) {
  if (!nodes || !origin || !h || !laser || !p || !F || nodes[0] < 2 || nodes[1] < 2 || nodes[2] < 2)
    return GM_ERR_ARG;
  const double r = p->laser_radius, d = p->laser_depth;
  const double rc = 1.0 / (r * sqrt(M_PI)), dc = 1.0 / (d * sqrt(M_PI));
  const double src_c = 6.0 * sqrt(3.0) * p->laser_eta * rc * rc * dc * (h[0] * h[1] * h[2] / 8.0);
  const long long n = (long long)nodes[0] * nodes[1] * nodes[2];
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == GM_F32)
    gm::fine_source_kernel<float><<<gm::lgrid(n), 256, 0, st>>>(nodes[0], nodes[1], nodes[2], origin[0], origin[1],
                                                                 origin[2], h[0], h[1], h[2], laser, r * r, d * d,
                                                                 src_c, (float*)F);
  else if (dtype == GM_F64)
    gm::fine_source_kernel<double><<<gm::lgrid(n), 256, 0, st>>>(nodes[0], nodes[1], nodes[2], origin[0], origin[1],
                                                                  origin[2], h[0], h[1], h[2], laser, r * r, d * d,
                                                                  src_c, (double*)F);
  else
    return GM_ERR_ARG;
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_fine_source_tables(int dtype, const int nodes[3], const double origin[3], const double h[3],
                                     const double* rows, int nrows, const gm_props* p, void* tab, void* stream) {
  if (!nodes || !origin || !h || !rows || !p || !tab || nrows < 1 || nodes[0] < 2 || nodes[1] < 2 || nodes[2] < 2)
    return GM_ERR_ARG;
  const double r = p->laser_radius, d = p->laser_depth;
  const double rc = 1.0 / (r * sqrt(M_PI)), dc = 1.0 / (d * sqrt(M_PI));
  const double src_c = 6.0 * sqrt(3.0) * p->laser_eta * rc * rc * dc * (h[0] * h[1] * h[2] / 8.0);
  const double ir2 = 1.0 / (r * r), id2 = 1.0 / (d * d);
  const long long n = (long long)nrows * (nodes[0] + nodes[1] + nodes[2]);
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == GM_F32)
    gm::fine_source_tables_kernel<float><<<gm::lgrid(n), 256, 0, st>>>(
        nodes[0], nodes[1], nodes[2], origin[0], origin[1], origin[2], (float)h[0], (float)h[1], (float)h[2], rows,
        nrows, (float)ir2, (float)id2, src_c, (float*)tab);
  else if (dtype == GM_F64)
    gm::fine_source_tables_kernel<double><<<gm::lgrid(n), 256, 0, st>>>(
        nodes[0], nodes[1], nodes[2], origin[0], origin[1], origin[2], h[0], h[1], h[2], rows, nrows, ir2, id2, src_c,
        (double*)tab);
  else
    return GM_ERR_ARG;
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_surface_flux(int dtype, const int nodes[3], const double h[3], int ne_planes, const void* T,
                               const gm_props* p, void* F, void* stream) {
  if (!nodes || !h || !T || !p || !F || nodes[0] < 2 || nodes[1] < 2 || ne_planes < 1 || ne_planes > nodes[2] - 1)
    return GM_ERR_ARG;
  const long long nxy = (long long)nodes[0] * nodes[1];
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == GM_F32)
    gm::surface_kernel<float><<<gm::lgrid(nxy), 256, 0, st>>>(nodes[0], nodes[1], ne_planes, h[0], h[1],
                                                               (const float*)T, (float*)F, gm::make_props<float>(*p));
  else if (dtype == GM_F64)
    gm::surface_kernel<double><<<gm::lgrid(nxy), 256, 0, st>>>(nodes[0], nodes[1], ne_planes, h[0], h[1],
                                                                (const double*)T, (double*)F,
                                                                gm::make_props<double>(*p));
  else
    return GM_ERR_ARG;
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}
