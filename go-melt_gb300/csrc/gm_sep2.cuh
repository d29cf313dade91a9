// Two fine Level-3 steps in one launch of the separable step (temporal
// blocking in the register ring).  Included by gm_level.cu after sep_body,
// whose LevelK, feature flags and surface-flux helper it uses.
//
// A warp owns 28 node columns (lanes 2..29; lanes 0, 1, 30, 31 are the x halo
// of the two steps) and BYT output rows, and marches a z-chunk of output
// planes.  Per node plane q it computes the first step's values S1(q) on its
// BYT + 2 strip rows and lanes 1..30 from the input planes q-1, q, q+1 (BYT + 4
// rows held in a register ring), then the second step's values of plane q-1
// from S1(q-2), S1(q-1), S1(q), with the arithmetic of the one-step kernel in
// the same order, so the result equals two one-step launches bit for bit.
// The first step's values stay in registers: per node and two steps the launch
// reads T and the phase byte once and writes them once.  Dirichlet nodes take
// the blended ring value of each step (clamped, as the one-step kernel writes
// them); the top plane (one-sided z operators, surface flux of each step's
// temperature) is computed by a z-slice of CTAs of its own that outputs the
// two highest planes, and the Dirichlet nodes by another.
#pragma once

namespace gm {

constexpr int SEP2_TILE = 28;  // output node columns of a warp
constexpr int SEP2_ZMAX = 30;  // output planes a CTA marches (its first-step planes, two more, one z factor a lane)

// Marching chunks of output planes 1 .. ntop-2 (the top slice outputs ntop-1 and ntop).
__host__ __device__ inline int sep2_march_chunks(int ntop, int zc) { return ntop > 2 ? cdiv(ntop - 2, zc) : 0; }

// 256-thread CTAs: at most 128 registers a thread (FP32, 1 or 2 rows), else 255
template <typename real, int BYT>
constexpr int sep2_min_blocks() {
  return sizeof(real) != 4 ? 1 : (BYT == 4 ? 1 : 2);
}

// The second step's per-step inputs (the first step's are in LevelK).
template <typename real>
struct Step2 {
  const double* dt;
  const real* src_tab;
  real bc_alpha, bc_beta;
};

// K.T of the NR middle rows of an (NR + 2)-row strip column at one plane
// (the one-step kernel's z, y and x stencils in its order of operations).
// TOP: one-sided z operators (Tp unused).  Every lane of the warp calls it.
template <typename real, int NR, bool TOP>
__device__ __forceinline__ RegCol<real, NR> sep_kt(const RegCol<real, NR + 2> Tm, const RegCol<real, NR + 2> T0,
                                                   const RegCol<real, NR + 2> Tp, real a1, real b1, real b2) {
  constexpr unsigned FULL = 0xffffffffu;
  real Zm[NR + 2], Zk[NR + 2];
#pragma unroll
  for (int i = 0; i < NR + 2; ++i) {
    if (TOP) {
      Zm[i] = rfma((real)2, T0.v[i], Tm.v[i]);
      Zk[i] = rsub(T0.v[i], Tm.v[i]);
    } else {
      const real s = radd(Tm.v[i], Tp.v[i]);
      Zm[i] = rfma((real)4, T0.v[i], s);
      Zk[i] = rfma((real)2, T0.v[i], -s);
    }
  }
  RegCol<real, NR> kt;
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    const int i = r + 1;
    const real u = radd(Zm[i - 1], Zm[i + 1]);
    const real w = radd(Zk[i - 1], Zk[i + 1]);
    const real A = rmul(a1, rfma((real)4, Zm[i], u));
    const real B = rfma(b1, rfma((real)2, Zm[i], -u), rmul(b2, rfma((real)4, Zk[i], w)));
    const real D = rsub(B, A);
    const real Dl = __shfl_up_sync(FULL, D, 1), Dr = __shfl_down_sync(FULL, D, 1);
    kt.v[r] = radd(rfma((real)2, A, rmul((real)4, B)), radd(Dl, Dr));
  }
  return kt;
}

// One CTA of the two-step launch: x-tile bx, strip group by, z-slice bz of a
// (gx, gy, ring_z + 1) grid; z-slice ring_z - 1 outputs the two top planes and
// ring_z the Dirichlet nodes.  Level-3 constant-property features only
// (laser factors from tables, surface flux, clamp, ring arrays, phase in and
// out; melt time with LF_ACCUM), every node at or below the top plane.
template <typename real, int BYT, int FL>
__device__ __forceinline__ void sep2_body(const LevelK<real>& a, const Step2<real>& b2, int bx, int by, int bz,
                                          int ring_z) {
  constexpr int RY1 = BYT + 2;  // first-step strip rows y0-1 .. y0+BYT
  constexpr int RY0 = BYT + 4;  // input strip rows y0-2 .. y0+BYT+1
  constexpr unsigned FULL = 0xffffffffu;
  constexpr bool hAcc = (FL & LF_ACCUM) != 0;
  static_assert((FL & ~LF_ACCUM) == (LF_L3 | LF_CONST), "Level-3 constant-property variants");

  const int nx = a.nx, ny = a.ny, nz = a.nz, nxy = nx * ny;
  const int lane = threadIdx.x & 31;
  const int x = bx * SEP2_TILE - 2 + lane;
  const int y0 = (by * (blockDim.x >> 5) + (threadIdx.x >> 5)) * BYT;
  const int ntop = a.ne_planes;  // nz - 1
  const Props<real>& P = a.p;
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  __shared__ real s_in[2];
  if (threadIdx.x == 0) {
    s_in[0] = (real)(*a.dt);
    s_in[1] = (real)(*b2.dt);
  }
  __syncthreads();
  const real dt1 = s_in[0], dt2 = s_in[1];
  const int subs = a.substrate > (long long)nxy * nz ? nxy * nz : (int)a.substrate;
  const bool xin = x >= 0 && x < nx;
  const bool out_x = lane >= 2 && lane < 2 + SEP2_TILE && x < nx;
  const bool ring_x = x == 0 || x == nx - 1;

  bool bad = false;  // a new value non-finite or above 1e5 K (before the clamp)
  auto report = [&]() {
    if (bad && a.status) atomicOr(a.status, GM_STATUS_BAD_T);
  };
  // phase bits after a step from the bits before it and the step's start temperature
  auto phase_after = [&](uint32_t ph, real Told, int id) -> uint32_t {
    const bool s2 = Told >= P.T_liquidus;
    const bool s1 = (ph & PH_S1) || s2 || id < subs;
    return (s1 ? PH_S1 : 0u) | (s2 ? PH_S2 : 0u);
  };
  // melt-time update of one step at a node (unchanged where not liquid)
  auto melt = [&](bool s2, bool prev2, real dt, real& acc, real& mac) {
    if (s2) {
      const real racc = prev2 ? (real)0 : acc;
      mac = fmax(racc, mac);
      acc = rsub(radd(acc, dt), racc);
    }
  };
  // Output of node id after both steps: Tn the second step's new value
  // (before the clamp), S1v the first step's (clamped), T0 the input, ph the
  // input phase byte, cAcc / cMacc its accumulators (read where liquid).
  auto finish2 = [&](int id, real Tn, real S1v, real T0, uint32_t ph, real cAcc, real cMacc) {
    bad = bad || !(Tn <= (real)1e5);
    Tn = fmax(Tn, P.T_amb);
    a.T_out[id] = Tn;
    const uint32_t p1 = phase_after(ph, T0, id);
    const uint32_t p2 = phase_after(p1, S1v, id);
    a.ph_out[id] = (uint8_t)p2;
    if (hAcc) {
      const bool s2a = (p1 & PH_S2) != 0, s2b = (p2 & PH_S2) != 0;
      if (s2a || s2b) {
        melt(s2a, (ph & PH_S2) != 0, dt1, cAcc, cMacc);
        melt(s2b, s2a, dt2, cAcc, cMacc);
        a.max_accum[id] = cMacc;
        a.accum[id] = cAcc;
      }
    }
  };

  if (bz == ring_z) {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    // ---- Dirichlet nodes: the bottom plane, then the x/y ring of planes
    // 1..nz-1 (the one-step kernel's enumeration) ----
    const int perim = 2 * nx + 2 * (ny - 2);
    const unsigned nring = (unsigned)(nxy + (nz - 1) * perim);
    const long long t0 = ((long long)by * gridDim.x + bx) * blockDim.x + threadIdx.x;
    if (t0 >= nring) return;
    const unsigned nthr = (unsigned)min((long long)gridDim.x * gridDim.y * blockDim.x, (long long)nring);
#pragma unroll 2
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
      const real bn = a.bc_new[id], bo = a.bc_old[id];
      const real T0 = a.T_in[id];
      const uint32_t ph = a.ph_in[id];
      real n1 = rfma(a.bc_alpha, bn, rmul(a.bc_beta, bo));
      bad = bad || !(n1 <= (real)1e5);
      n1 = fmax(n1, P.T_amb);
      const real n2 = rfma(b2.bc_alpha, bn, rmul(b2.bc_beta, bo));
      const bool liq = hAcc && (T0 >= P.T_liquidus || n1 >= P.T_liquidus);
      finish2(id, n2, n1, T0, ph, liq ? a.accum[id] : (real)0, liq ? a.max_accum[id] : (real)0);
    }
    report();
    return;
  }

  // z-slice ring_z - 1 outputs planes ntop-1 and ntop, the others a chunk of 1 .. ntop-2
  const bool top_slice = bz == ring_z - 1;
  const int Z0 = top_slice ? ntop - 1 : 1 + bz * a.zchunk;
  const int Z1 = top_slice ? ntop + 1 : min(ntop - 1, Z0 + a.zchunk);
  const real a1 = a.sa1, b1 = a.sb1, b2c = a.sb2;
  const real minv1 = dt1 / a.smass, minv2 = dt2 / a.smass;

  // laser factors: x times the rows' y factors per step; lane l keeps the
  // first step's z factor of plane Z0-1+l and the second's of plane Z0+l
  real sxy1[RY1], sxy2[BYT], szl1 = 0, szl2 = 0;
  {
    const real* t1 = a.src_tab;
    const real* t2 = b2.src_tab;
    const real sx1 = xin ? t1[x] : (real)0, sx2 = xin ? t2[x] : (real)0;
    const int yl = y0 - 1 + lane;
    const real sy1 = (lane < RY1 && yl >= 0 && yl < ny) ? t1[nx + yl] : (real)0;
    const real sy2 = (lane < BYT && y0 + lane < ny) ? t2[nx + y0 + lane] : (real)0;
#pragma unroll
    for (int j = 0; j < RY1; ++j) sxy1[j] = rmul(sx1, __shfl_sync(FULL, sy1, j));
#pragma unroll
    for (int r = 0; r < BYT; ++r) sxy2[r] = rmul(sx2, __shfl_sync(FULL, sy2, r));
    const int z1 = Z0 - 1 + lane, z2 = Z0 + lane;
    if (z1 >= 0 && z1 < nz && z1 <= Z1) szl1 = t1[nx + ny + z1];
    if (z2 < Z1) szl2 = t2[nx + ny + z2];
  }
  asm volatile("griddepcontrol.wait;" ::: "memory");

  // rows this warp outputs (not on the y ring, inside the grid)
  bool row_out[BYT];
#pragma unroll
  for (int r = 0; r < BYT; ++r) row_out[r] = out_x && !ring_x && y0 + r > 0 && y0 + r < ny - 1;
  // a Dirichlet node in the first-step strip of an interior plane (x/y ring)
  bool dir_row[RY1];
  bool has_ring = false;
#pragma unroll
  for (int j = 0; j < RY1; ++j) {
    const int y = y0 - 1 + j;
    dir_row[j] = xin && y >= 0 && y < ny && (ring_x || y == 0 || y == ny - 1);
    has_ring = has_ring || dir_row[j];
  }
  has_ring = __any_sync(FULL, has_ring);

  const real* Tcol = a.T_in + (x + (y0 - 2) * nx);  // input strip row 0 of plane 0 (dereferenced inside the grid)
  auto load_plane = [&](real(&dst)[RY0], int pl) {
    const bool ok = xin && pl >= 0 && pl < nz;
#pragma unroll
    for (int i = 0; i < RY0; ++i) {
      const int y = y0 - 2 + i;
      dst[i] = (ok && y >= 0 && y < ny) ? Tcol[i * nx + pl * nxy] : (real)0;
    }
  };
  // ring values of the first-step strip at plane pl (Dirichlet nodes only;
  // every node of plane 0)
  real rbn[RY1], rbo[RY1];
  auto load_ring = [&](int pl) {
#pragma unroll
    for (int j = 0; j < RY1; ++j) {
      rbn[j] = rbo[j] = 0;
      const int y = y0 - 1 + j;
      if (dir_row[j] || (pl == 0 && xin && y >= 0 && y < ny)) {
        const int id = x + y * nx + pl * nxy;
        rbn[j] = a.bc_new[id];
        rbo[j] = a.bc_old[id];
      }
    }
  };
  // phase bytes of an output plane, loaded two planes ahead
  uint32_t nph[3][BYT];
  auto prefetch_ph = [&](auto slot_c, int pl) {
    constexpr int S = decltype(slot_c)::value;
#pragma unroll
    for (int r = 0; r < BYT; ++r) {
      nph[S][r] = 0;
      if (row_out[r] && pl < Z1) nph[S][r] = a.ph_in[x + (y0 + r) * nx + pl * nxy];
    }
  };
  // melt-time accumulators of the output nodes of plane pl that are liquid
  // at the start of either step (T0: input rows, S: first-step rows)
  real nacc[2][BYT], nmac[2][BYT];
  auto prefetch_acc = [&](auto slot_c, int pl, const RegCol<real, RY0> T0, const RegCol<real, RY1> S) {
    constexpr int SL = decltype(slot_c)::value;
    bool liq[BYT], any = false;
#pragma unroll
    for (int r = 0; r < BYT; ++r) {
      liq[r] = row_out[r] && pl >= Z0 && pl < Z1 && (T0.v[r + 2] >= P.T_liquidus || S.v[r + 1] >= P.T_liquidus);
      any = any || liq[r];
      nacc[SL][r] = nmac[SL][r] = 0;
    }
    if (__any_sync(FULL, any)) {
#pragma unroll
      for (int r = 0; r < BYT; ++r)
        if (liq[r]) {
          const int id = x + (y0 + r) * nx + pl * nxy;
          nacc[SL][r] = a.accum[id];
          nmac[SL][r] = a.max_accum[id];
        }
    }
  };

  // First step at plane q into S: the stencil (TOP: one-sided, plus the surface
  // flux `surf`) where q is interior, the blended ring value at Dirichlet nodes.
  // Values of the nodes this warp outputs (planes Z0..Z1-1) are checked.
  auto step1 = [&](auto top_c, int q, const RegCol<real, RY0> Tm, const RegCol<real, RY0> T0,
                   const RegCol<real, RY0> Tp, const RegCol<real, RY1> surf) {
    constexpr bool TOP = decltype(top_c)::value;
    RegCol<real, RY1> S;
    const real sz = __shfl_sync(FULL, szl1, q - (Z0 - 1));
    const RegCol<real, RY1> kt = sep_kt<real, RY1, TOP>(Tm, T0, Tp, a1, b1, b2c);
    const real mi = TOP ? (real)2 * minv1 : minv1;
    const bool own = q >= Z0 && q < Z1;
#pragma unroll
    for (int j = 0; j < RY1; ++j) {
      real Rt = -kt.v[j];
      Rt = rfma(sxy1[j], sz, Rt);
      if (TOP) Rt = radd(Rt, surf.v[j]);
      real Tn = rfma(Rt, mi, T0.v[j + 1]);
      if (own && j >= 1 && j <= BYT && row_out[j - 1]) bad = bad || !(Tn <= (real)1e5);
      Tn = fmax(Tn, P.T_amb);
      if (has_ring && dir_row[j]) Tn = fmax(rfma(a.bc_alpha, rbn[j], rmul(a.bc_beta, rbo[j])), P.T_amb);
      S.v[j] = Tn;
    }
    return S;
  };
  // the first step's values of Dirichlet plane 0
  auto step1_bottom = [&]() {
    RegCol<real, RY1> S;
#pragma unroll
    for (int j = 0; j < RY1; ++j) S.v[j] = fmax(rfma(a.bc_alpha, rbn[j], rmul(a.bc_beta, rbo[j])), P.T_amb);
    return S;
  };
  // Second step at output plane p from first-step planes p-1, p, p+1 (TOP:
  // one-sided, surface flux `surf` of the first step's top plane).
  auto step2 = [&](auto top_c, int p, const RegCol<real, RY1> Sm, const RegCol<real, RY1> S0,
                   const RegCol<real, RY1> Sp, const RegCol<real, BYT> surf, const RegCol<real, RY0> T0,
                   const RegCol<uint32_t, BYT> ph, const RegCol<real, BYT> acc, const RegCol<real, BYT> mac) {
    constexpr bool TOP = decltype(top_c)::value;
    const real sz = __shfl_sync(FULL, szl2, p - Z0);
    const RegCol<real, BYT> kt = sep_kt<real, BYT, TOP>(Sm, S0, Sp, a1, b1, b2c);
    const real mi = TOP ? (real)2 * minv2 : minv2;
#pragma unroll
    for (int r = 0; r < BYT; ++r) {
      if (!row_out[r]) continue;
      real Rt = -kt.v[r];
      Rt = rfma(sxy2[r], sz, Rt);
      if (TOP) Rt = radd(Rt, surf.v[r]);
      const real Tn = rfma(Rt, mi, S0.v[r + 1]);
      finish2(x + (y0 + r) * nx + p * nxy, Tn, S0.v[r + 1], T0.v[r + 2], ph.v[r], acc.v[r], mac.v[r]);
    }
  };

  // register arrays passed by value to the steps
  auto col0 = [&](const real* c) {
    RegCol<real, RY0> o;
#pragma unroll
    for (int i = 0; i < RY0; ++i) o.v[i] = c[i];
    return o;
  };
  auto col1 = [&](const real* c) {
    RegCol<real, RY1> o;
#pragma unroll
    for (int j = 0; j < RY1; ++j) o.v[j] = c[j];
    return o;
  };
  auto rows_of = [&](const real* c) {
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
  const RegCol<real, RY1> nosurf1 = {};
  const RegCol<real, BYT> nosurf2 = {};

  if (top_slice) {
    if (ntop < 2) return;
    // input planes ntop-3 .. ntop, first-step planes ntop-2 .. ntop, output planes ntop-1, ntop
    real T3[RY0], T2[RY0], T1[RY0], T0[RY0];
    load_plane(T3, ntop - 3);
    load_plane(T2, ntop - 2);
    load_plane(T1, ntop - 1);
    load_plane(T0, ntop);
    prefetch_ph(std::integral_constant<int, 0>(), ntop - 1);
    prefetch_ph(std::integral_constant<int, 1>(), ntop);
    load_ring(ntop - 2);
    const RegCol<real, RY1> Sa = (ntop - 2 == 0) ? step1_bottom()
                                                 : step1(std::false_type(), ntop - 2, col0(T3), col0(T2), col0(T1), nosurf1);
    load_ring(ntop - 1);
    const RegCol<real, RY1> Sb = step1(std::false_type(), ntop - 1, col0(T2), col0(T1), col0(T0), nosurf1);
    load_ring(ntop);
    const RegCol<real, RY1> sf1 = sep_surface<real, RY1>(P, a.w2, x, nx, y0 - 1, ny, col0(T0));
    const RegCol<real, RY1> Sc = step1(std::true_type(), ntop, col0(T1), col0(T0), col0(T0), sf1);
    if (hAcc) {
      prefetch_acc(std::integral_constant<int, 0>(), ntop - 1, col0(T1), Sb);
      prefetch_acc(std::integral_constant<int, 1>(), ntop, col0(T0), Sc);
    }
    step2(std::false_type(), ntop - 1, Sa, Sb, Sc, nosurf2, col0(T1), phase_of(nph[0]), rows_of(nacc[0]),
          rows_of(nmac[0]));
    const RegCol<real, BYT> sf2 = sep_surface<real, BYT>(P, a.w2, x, nx, y0, ny, Sc);
    step2(std::true_type(), ntop, Sb, Sc, Sc, sf2, col0(T0), phase_of(nph[1]), rows_of(nacc[1]), rows_of(nmac[1]));
    report();
    return;
  }

  // ---- marching chunk: iteration k computes the first step at plane
  // q = Z0-1+k and the second step at plane q-1 (k >= 2) ----
  // input plane t in slot (t - Z0 + 2) % 6, first-step plane q in slot
  // (q - Z0 + 1) % 3, phase of output plane p in slot (p - Z0) % 3,
  // accumulators of output plane p in slot (p - Z0 + 1) & 1
  real Tr[6][RY0];
  real Sr[3][RY1];
  load_plane(Tr[0], Z0 - 2);
  load_plane(Tr[1], Z0 - 1);
  load_plane(Tr[2], Z0);
  load_plane(Tr[3], Z0 + 1);
  if (has_ring || Z0 - 1 == 0) load_ring(Z0 - 1);
  const int nk = Z1 - Z0 + 2;

  auto body = [&](auto par, int k) {
    constexpr int PAR = decltype(par)::value;
    const int q = Z0 - 1 + k;
    if (q + 3 <= Z1 + 1) load_plane(Tr[(PAR + 4) % 6], q + 3);
    prefetch_ph(std::integral_constant<int, PAR % 3>(), Z0 + k);
    const RegCol<real, RY1> S =
        (q == 0) ? step1_bottom()
                 : step1(std::false_type(), q, col0(Tr[PAR % 6]), col0(Tr[(PAR + 1) % 6]), col0(Tr[(PAR + 2) % 6]),
                         nosurf1);
#pragma unroll
    for (int j = 0; j < RY1; ++j) Sr[PAR % 3][j] = S.v[j];
    if (has_ring && q + 1 <= Z1) load_ring(q + 1);
    if (hAcc) prefetch_acc(std::integral_constant<int, PAR & 1>(), q, col0(Tr[(PAR + 1) % 6]), S);
    if (k >= 2)
      step2(std::false_type(), q - 1, col1(Sr[(PAR + 1) % 3]), col1(Sr[(PAR + 2) % 3]), S, nosurf2,
            col0(Tr[PAR % 6]), phase_of(nph[(PAR + 1) % 3]), rows_of(nacc[(PAR + 1) & 1]),
            rows_of(nmac[(PAR + 1) & 1]));
  };

  for (int k = 0; k < nk; k += 6) {
    body(std::integral_constant<int, 0>(), k);
    if (k + 1 < nk) body(std::integral_constant<int, 1>(), k + 1);
    if (k + 2 < nk) body(std::integral_constant<int, 2>(), k + 2);
    if (k + 3 < nk) body(std::integral_constant<int, 3>(), k + 3);
    if (k + 4 < nk) body(std::integral_constant<int, 4>(), k + 4);
    if (k + 5 < nk) body(std::integral_constant<int, 5>(), k + 5);
  }
  report();
}

template <typename real, int BYT, int FL>
__global__ void __launch_bounds__(256, sep2_min_blocks<real, BYT>())
    level_sep2_kernel(const LevelK<real> a, const Step2<real> b) {
  sep2_body<real, BYT, FL>(a, b, blockIdx.x, blockIdx.y, blockIdx.z, gridDim.z - 1);
}

}  // namespace gm
