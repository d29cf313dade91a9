// Native orchestration of the multilevel step: the whole subcycleGOMELT
// (go_melt/computeFunctions.py:3224-3632) issued from C++ on one stream.
//
// Sequence (N2 Level-2 steps of N3 Level-3 steps each, predictor then
// corrector, as the reference's two lax.scan passes):
//   Level-1 S1 from Level 2 at the overlap (:3272-3278)
//   Level-1 RHS = source over all rows + T' fluxes of L3 and L2 (:3285-3292)
//   Level-1 predictor (:3294-3305)
//   pass 1: per Level-2 step: Level-2 RHS (source of its rows + L3 T' flux),
//           Level-2 solve with the blended Level-1 ring, N3 Level-3 solves with
//           the blended Level-2 ring, restriction + T'3 (:3307-3430); the two
//           coarse fields of each blend are prolongated onto the ring once
//           (per pass for Level 2, per Level-2 step for Level 3)
//   T'2, Level-1 mass terms, Level-1 corrector (:3432-3456)
//   pass 2: as pass 1 from the saved state, plus the Level-2 mass term and the
//           Level-3 melt-time update (:3458-3622)
//   final T'2 / Level-1 restriction, Level-0 S1 store (:3625-3630)
#include <cuda_runtime.h>
#include <string.h>

#include <vector>

#include "gm_common.cuh"
#include "gomelt.h"

namespace {

struct Ctx {
  const gm_subcycle_plan* p;
  const gm_props* pr;
  void* st;
  size_t esz;
  int rc = GM_OK;
  int persist = 0;        // Level-3 steps of a Level-2 step as one launch: 1 tiles in shared memory, 2 grid steps
  unsigned pbase = 0;     // flag value at the next persistent launch (mode 1)
  int plaunch = 0;        // persistent launches issued in this call (mode 2: counter index)
  int pairs = 0;          // Level-3 fine steps two at a time (gm_level_step2)
};

inline char* at(void* base, long long elems, size_t esz) { return (char*)base + elems * (long long)esz; }
inline long long nn(const gm_window& w) { return (long long)w.nodes[0] * w.nodes[1] * w.nodes[2]; }

#define GM_TRY(expr)             \
  do {                           \
    if (c.rc == GM_OK) {         \
      int _r = (expr);           \
      if (_r != GM_OK) c.rc = _r; \
    }                            \
  } while (0)

gm_level_args level_args(Ctx& c, const gm_window& w, int ne_planes, const void* Tin, void* Tout, const double* dt,
                         const uint8_t* phin, uint8_t* phout, const void* rhs, const int lo[3], const int n[3],
                         const double* laser, int bc_mode, const gm_map3* map, const void* bnew, const void* bold,
                         double alpha, void* acc, void* macc, const void* src_tab) {
  const gm_subcycle_plan& p = *c.p;
  gm_level_args a;
  memset(&a, 0, sizeof(a));
  a.dtype = p.dtype;
  a.nx = w.nodes[0];
  a.ny = w.nodes[1];
  a.nz = w.nodes[2];
  for (int d = 0; d < 3; ++d) {
    a.h[d] = w.h[d];
    a.origin[d] = w.origin[d];
  }
  a.ne_planes = ne_planes;
  a.dt = dt;
  a.T_in = Tin;
  a.T_out = Tout;
  a.ph_in = phin;
  a.ph_out = phout;
  a.substrate = w.substrate;
  if (rhs) {
    a.rhs_box = rhs;
    for (int d = 0; d < 3; ++d) {
      a.box[2 * d] = lo[d];
      a.box[2 * d + 1] = lo[d] + n[d];
    }
  }
  a.laser = laser;
  a.surface = 1;
  a.bc_mode = bc_mode;
  if (bc_mode == 1) {
    for (int i = 0; i < 5; ++i) a.face[i] = p.face[i];
    a.inactive_amb = 1;
  } else if (bc_mode == 2 || bc_mode == 3) {
    a.bc_new = bnew;
    a.bc_old = bold;
    a.bc_alpha = alpha;
    a.bc_beta = 1.0 - alpha;
    if (map) a.bc_map = *map;
  }
  a.clamp = 1;
  a.accum = acc;
  a.max_accum = macc;
  a.zchunk = p.zchunk;
  a.pdl = p.pdl;  // dt, the laser row and its factor table are never written by the kernels before it
  a.src_tab = src_tab;
  a.status = p.pstatus;  // non-finite or out-of-range results of any level step
  return a;
}

void level(Ctx& c, const gm_window& w, int ne_planes, const void* Tin, void* Tout, const double* dt,
           const uint8_t* phin, uint8_t* phout, const void* rhs, const int lo[3], const int n[3],
           const double* laser, int bc_mode, const gm_map3* map, const void* bnew, const void* bold, double alpha,
           void* acc, void* macc, const void* src_tab = nullptr) {
  const gm_level_args a = level_args(c, w, ne_planes, Tin, Tout, dt, phin, phout, rhs, lo, n, laser, bc_mode, map,
                                     bnew, bold, alpha, acc, macc, src_tab);
  GM_TRY(gm_level_step(&a, c.pr, c.st));
}

void couple(Ctx& c, const gm_couple_geom& g, const gm_window& fine, void* out, const int lo[3], const int n[3],
            const void* Tp, const void* dTa, const void* dTb, const double* dt, const void* base = nullptr) {
  const gm_subcycle_plan& p = *c.p;
  gm_couple_args a;
  memset(&a, 0, sizeof(a));
  a.dtype = p.dtype;
  a.geom = g;
  for (int d = 0; d < 3; ++d) {
    a.fine_nodes[d] = fine.nodes[d];
    a.fine_h[d] = fine.h[d];
    a.out_lo[d] = lo[d];
    a.out_n[d] = n[d];
  }
  a.T = fine.T;
  a.ph = fine.ph;
  a.substrate = fine.substrate;
  a.Tp = Tp;
  a.dTa = dTa;
  a.dTb = dTb;
  a.dt = dt;
  a.out = out;
  a.scale = 1.0;
  a.partials = p.partials;
  a.partials_cap = p.partials_cap;
  a.base = base;
  GM_TRY(gm_couple(&a, c.pr, c.st));
}

// couple() reads the fine level's T/phase from the window; the passes use
// carried fields instead, so this variant takes them explicitly.
void couple_fields(Ctx& c, const gm_couple_geom& g, const gm_window& fine, const void* T, const uint8_t* ph,
                   void* out, const int lo[3], const int n[3], const void* Tp, const void* dTa, const void* dTb,
                   const double* dt, const void* base = nullptr) {
  gm_window w = fine;
  w.T = (void*)T;
  w.ph = (uint8_t*)ph;
  couple(c, g, w, out, lo, n, Tp, dTa, dTb, dt, base);
}

void source(Ctx& c, const gm_couple_geom& g, const double* const xq[3], const double* rows, int npos, void* out,
            const int lo[3], const int n[3], int ngroups = 1, long long group_stride = 0) {
  const gm_subcycle_plan& p = *c.p;
  gm_coarse_source_args a;
  memset(&a, 0, sizeof(a));
  a.dtype = p.dtype;
  a.geom = g;
  a.npos = npos;
  a.rows = rows;
  for (int d = 0; d < 3; ++d) {
    a.xq[d] = xq[d];
    a.out_lo[d] = lo[d];
    a.out_n[d] = n[d];
  }
  a.fine_wq = p.L3.h[0] * p.L3.h[1] * p.L3.h[2] / 8.0;
  a.out = out;
  a.scratch = p.src_scratch;
  a.scratch_cap = p.src_cap;
  a.ngroups = ngroups;
  a.out_group_stride = group_stride;
  GM_TRY(gm_coarse_source(&a, c.pr, c.st));
}

// getNewTprime (:2060-2099): restrict the fine field into coarse_T, then
// T' = T_f - I(T_c).
void new_tprime(Ctx& c, const gm_map3& rmap, const int* const idx[3], const gm_window& coarse, const gm_map3& cmap,
                const gm_window& fine, const void* fineT, void* coarseT, void* outTp, const int* const inj[9]) {
  const gm_subcycle_plan& p = *c.p;
  if (inj[0]) {  // the restriction is an injection: one pass
    gm_tprime_args t;
    memset(&t, 0, sizeof(t));
    t.dtype = p.dtype;
    for (int d = 0; d < 3; ++d) {
      t.n[d] = fine.nodes[d];
      t.cf0[d] = inj[d];
      t.cf1[d] = inj[3 + d];
      t.c_of_f[d] = inj[6 + d];
    }
    t.cmap = cmap;
    t.cnx = coarse.nodes[0];
    t.cny = coarse.nodes[1];
    t.fine = fineT;
    t.coarse = coarseT;
    t.out = outTp;
    GM_TRY(gm_tprime_inject(&t, c.st));
    return;
  }
  gm_restrict_args r;
  memset(&r, 0, sizeof(r));
  r.dtype = p.dtype;
  for (int d = 0; d < 3; ++d) {
    r.n[d] = rmap.n[d];
    r.cidx[d] = idx[d];
  }
  r.map = rmap;
  r.cnx = coarse.nodes[0];
  r.cny = coarse.nodes[1];
  r.fine = fineT;
  r.coarse = coarseT;
  GM_TRY(gm_restrict(&r, c.st));
  gm_interp_args a;
  memset(&a, 0, sizeof(a));
  a.dtype = p.dtype;
  for (int d = 0; d < 3; ++d) a.n[d] = fine.nodes[d];
  a.nterms = 1;
  a.map[0] = cmap;
  a.src[0] = coarseT;
  a.coef[0] = -1.0;
  a.base = fineT;
  a.out = outTp;
  GM_TRY(gm_interp(&a, c.st));
}

void memzero(Ctx& c, void* ptr, long long elems) {
  if (c.rc != GM_OK) return;
  if (cudaMemsetAsync(ptr, 0, elems * c.esz, (cudaStream_t)c.st) != cudaSuccess) c.rc = GM_ERR_CUDA;
}

void copy(Ctx& c, void* dst, const void* src, long long bytes) {
  if (c.rc != GM_OK || dst == src) return;
  if (cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, (cudaStream_t)c.st) != cudaSuccess)
    c.rc = GM_ERR_CUDA;
}

// Both coarse fields of a blend prolongated onto a fine level's ring once
// (gm_ring_prolong); the level steps then use bc_mode 3.
void ring(Ctx& c, const gm_window& fine, const gm_map3& map, const void* A, const void* B, void* outA, void* outB) {
  gm_ring_args r;
  memset(&r, 0, sizeof(r));
  r.dtype = c.p->dtype;
  for (int d = 0; d < 3; ++d) r.nodes[d] = fine.nodes[d];
  r.map = map;
  r.srcA = A;
  r.srcB = B;
  r.outA = outA;
  r.outB = outB;
  GM_TRY(gm_ring_prolong(&r, c.st));
}

struct PassOut {
  void* T2;
  uint8_t* ph2;
  void* T3;
  uint8_t* ph3;
  void* Tp3;
};

// One pass over the N2 Level-2 steps (subcycleL2_Part1 / subcycleL2_Part2).
PassOut l2_pass(Ctx& c, const void* T1new, bool part2) {
  const gm_subcycle_plan& p = *c.p;
  const int N2 = p.N2, N3 = p.N3;
  const long long n3 = nn(p.L3);
  void* T2c = p.L2.T;
  uint8_t* ph2c = p.L2.ph;
  void* T3c = p.L3.T;
  uint8_t* ph3c = p.L3.ph;
  void* Tp3c = p.L3.Tp;
  const long long nrhs2 = (long long)p.rhs2_n[0] * p.rhs2_n[1] * p.rhs2_n[2];
  ring(c, p.L2, p.bc12, T1new, p.L1.T, p.ring2[0], p.ring2[1]);
  for (int l2 = 0; l2 < N2; ++l2) {
    void* hist_l2 = at(p.tp3hist, l2 * n3, c.esz);
    const double* dt2 = p.dts + 1 + l2;
    // rhs2 = the step's source (computed once for the call) + the coupling terms
    const void* src = at(p.src2, l2 * nrhs2, c.esz);
    if (part2)
      couple_fields(c, p.c32, p.L3, T3c, ph3c, p.rhs2, p.rhs2_lo, p.rhs2_n, Tp3c, hist_l2, Tp3c, dt2, src);
    else
      couple_fields(c, p.c32, p.L3, T3c, ph3c, p.rhs2, p.rhs2_lo, p.rhs2_n, Tp3c, nullptr, nullptr, nullptr, src);
    void* T2n = p.T2w[l2 % 2];
    uint8_t* ph2n = p.ph2w[l2 % 2];
    level(c, p.L2, p.L2.nodes[2] - 1, T2c, T2n, dt2, ph2c, ph2n, p.rhs2, p.rhs2_lo, p.rhs2_n, nullptr, 3, nullptr,
          p.ring2[0], p.ring2[1], (l2 + 1) / (double)N2, nullptr, nullptr);
    ring(c, p.L3, p.bc23, T2n, T2c, p.ring3[0], p.ring3[1]);
    if (c.persist == 2) {  // all N3 fine steps in one launch of the one-step kernel's body, grid barriers
      const int i0 = l2 * N3;
      const long long L3n = (long long)p.L3.nodes[0] + p.L3.nodes[1] + p.L3.nodes[2];
      gm_steps_args sa;
      memset(&sa, 0, sizeof(sa));
      sa.level = level_args(c, p.L3, p.L3.nodes[2] - 1, T3c, p.T3w[l2 % 2], p.rows + (long long)i0 * 7 + 5, ph3c,
                            p.ph3w[l2 % 2], nullptr, nullptr, nullptr, p.rows + (long long)i0 * 7, 3, nullptr,
                            p.ring3[0], p.ring3[1], 1.0 / N3, part2 ? p.acc3 : nullptr, part2 ? p.macc3 : nullptr,
                            at(p.src3tab, i0 * L3n, c.esz));
      sa.level.pdl = 0;
      sa.nsteps = N3;
      sa.nsub = N3;
      sa.rows = p.rows + (long long)i0 * 7;
      sa.src_tab = at(p.src3tab, i0 * L3n, c.esz);
      sa.tbuf[0] = p.xch3[0];
      sa.tbuf[1] = p.xch3[1];
      sa.counter = p.pflags + c.plaunch++;
      sa.base = 0;
      sa.status = p.pstatus;
      GM_TRY(gm_level3_steps(&sa, c.pr, c.st));
      T3c = sa.level.T_out;
      ph3c = sa.level.ph_out;
    } else if (c.persist == 1) {  // all N3 fine steps in one launch
      const int i0 = l2 * N3;
      const long long L3n = (long long)p.L3.nodes[0] + p.L3.nodes[1] + p.L3.nodes[2];
      gm_persist_args a;
      memset(&a, 0, sizeof(a));
      a.dtype = p.dtype;
      for (int d = 0; d < 3; ++d) {
        a.nodes[d] = p.L3.nodes[d];
        a.h[d] = p.L3.h[d];
      }
      a.nsteps = N3;
      a.nsub = N3;
      a.T_in = T3c;
      a.T_out = p.T3w[l2 % 2];
      a.ph_in = ph3c;
      a.ph_out = p.ph3w[l2 % 2];
      a.substrate = p.L3.substrate;
      a.ring_new = p.ring3[0];
      a.ring_old = p.ring3[1];
      a.src_tab = at(p.src3tab, i0 * L3n, c.esz);
      a.rows = p.rows + (long long)i0 * 7;
      a.accum = part2 ? p.acc3 : nullptr;
      a.max_accum = part2 ? p.macc3 : nullptr;
      a.xbuf[0] = p.xch3[0];
      a.xbuf[1] = p.xch3[1];
      a.flags = p.pflags;
      a.flags_cap = p.pflags_cap;
      a.base = c.pbase;
      a.status = p.pstatus;
      GM_TRY(gm_level3_persist(&a, c.pr, c.st));
      c.pbase += (unsigned)N3;
      T3c = a.T_out;
      ph3c = a.ph_out;
    }
    for (int l3 = 0; l3 < (c.persist ? 0 : N3);) {  // one launch a fine step, or one a pair of them
      const int i = l2 * N3 + l3;
      void* Tn = T3c == p.T3w[0] ? p.T3w[1] : p.T3w[0];
      uint8_t* phn = ph3c == p.ph3w[0] ? p.ph3w[1] : p.ph3w[0];
      const double* row = p.rows + (long long)i * 7;
      const long long L3n = (long long)p.L3.nodes[0] + p.L3.nodes[1] + p.L3.nodes[2];
      if (c.pairs && l3 + 1 < N3) {  // steps l3 and l3 + 1 in one launch
        gm_level2_args a2;
        memset(&a2, 0, sizeof(a2));
        a2.level = level_args(c, p.L3, p.L3.nodes[2] - 1, T3c, Tn, row + 5, ph3c, phn, nullptr, nullptr, nullptr, row,
                              3, nullptr, p.ring3[0], p.ring3[1], (l3 + 1) / (double)N3, part2 ? p.acc3 : nullptr,
                              part2 ? p.macc3 : nullptr, at(p.src3tab, i * L3n, c.esz));
        a2.dt2 = row + 7 + 5;
        a2.src_tab2 = at(p.src3tab, (i + 1) * L3n, c.esz);
        a2.bc_alpha2 = (l3 + 2) / (double)N3;
        a2.bc_beta2 = 1.0 - a2.bc_alpha2;
        GM_TRY(gm_level_step2(&a2, c.pr, c.st));
        l3 += 2;
      } else {
        level(c, p.L3, p.L3.nodes[2] - 1, T3c, Tn, row + 5, ph3c, phn, nullptr, nullptr, nullptr, row, 3, nullptr,
              p.ring3[0], p.ring3[1], (l3 + 1) / (double)N3, part2 ? p.acc3 : nullptr, part2 ? p.macc3 : nullptr,
              p.src3tab ? at(p.src3tab, i * L3n, c.esz) : nullptr);
        l3 += 1;
      }
      T3c = Tn;
      ph3c = phn;
    }
    void* Tp3n = part2 ? p.tp3w[l2 % 2] : hist_l2;
    new_tprime(c, p.r32, p.r32_idx, p.L2, p.bc23, p.L3, T3c, T2n, Tp3n, p.inj32);
    if (part2 && p.L2all) {
      copy(c, at(p.L2all, (long long)l2 * nn(p.L2), c.esz), T2n, nn(p.L2) * c.esz);
      copy(c, at(p.L3all, l2 * n3, c.esz), T3c, n3 * c.esz);
      copy(c, at(p.L3pall, l2 * n3, c.esz), Tp3n, n3 * c.esz);
    }
    Tp3c = Tp3n;
    T2c = T2n;
    ph2c = ph2n;
  }
  return PassOut{T2c, ph2c, T3c, ph3c, Tp3c};
}

bool plan_ok(const gm_subcycle_plan* p) {
  if (!p || p->N2 < 1 || p->N3 < 1 || !p->rows || !p->dts) return false;
  const gm_window* ws[3] = {&p->L1, &p->L2, &p->L3};
  for (auto w : ws)
    if (!w->T || !w->ph || w->nodes[0] < 2 || w->nodes[1] < 2 || w->nodes[2] < 2) return false;
  if (!p->L2.Tp || !p->L3.Tp || !p->acc3 || !p->macc3) return false;
  if (!p->T1p || !p->T1c || !p->T2w[0] || !p->T2w[1] || !p->T3w[0] || !p->T3w[1] || !p->tp3w[0] || !p->tp3w[1] ||
      !p->Tp2w || !p->rhs1 || !p->rhs2 || !p->tp3hist || !p->ph2w[0] || !p->ph2w[1] || !p->ph3w[0] || !p->ph3w[1] ||
      !p->partials || !p->src_scratch || !p->L0 || !p->ring2[0] || !p->ring2[1] || !p->ring3[0] || !p->ring3[1] ||
      !p->src2)
    return false;
  if ((p->L2all == nullptr) != (p->L3all == nullptr) || (p->L2all == nullptr) != (p->L3pall == nullptr)) return false;
  return true;
}

}  // namespace

namespace {

int subcycle_issue(const gm_subcycle_plan* p, const gm_props* props, void* stream) {
  Ctx c;
  c.p = p;
  c.pr = props;
  c.st = stream;
  c.esz = p->dtype == GM_F32 ? 4 : 8;
  const long long n1 = nn(p->L1), n2 = nn(p->L2), n3 = nn(p->L3);
  const long long nrhs1 = (long long)p->rhs1_n[0] * p->rhs1_n[1] * p->rhs1_n[2];

  // The Level-3 laser factors of the call, tabulated by an ordinarily
  // launched kernel that triggers no early launch: every kernel after it
  // starts once it has completed, so their prologues may read the table.
  if (p->src3tab)
    GM_TRY(gm_fine_source_tables(p->dtype, p->L3.nodes, p->L3.origin, p->L3.h, p->rows, p->N2 * p->N3, props,
                                 p->src3tab, stream));
  // persistent Level-3 steps: needs the factor table, the work buffers and a
  // constant-property material; the window must have a persistent shape
  const bool kconst = props->k_powder == props->k_bulk_a0 && props->k_fluid == props->k_bulk_a0 &&
                      props->k_bulk_a1 == 0.0 && props->cp_solid_a1 == 0.0 && props->cp_mushy == props->cp_solid_a0 &&
                      props->cp_fluid == props->cp_solid_a0;
  if (p->persist && p->src3tab && p->xch3[0] && p->xch3[1] && p->pflags && p->pstatus) {
    if (p->persist == 1) {
      int shp[4];
      const long long nf = gm_level3_persist_flags(p->L3.nodes);
      c.persist = (nf > 0 && nf <= p->pflags_cap && gm_level3_persist_shape(p->dtype, p->L3.nodes, shp) == GM_OK &&
                   kconst) ? 1 : 0;
    } else if (p->persist == 2) {
      c.persist = (kconst && p->pflags_cap >= 2LL * p->N2) ? 2 : 0;  // a barrier counter per launch
    }
    if (c.persist &&
        cudaMemsetAsync(p->pflags, 0, sizeof(unsigned) * p->pflags_cap, (cudaStream_t)stream) != cudaSuccess)
      return GM_ERR_CUDA;
  }
  // Level-3 fine steps two at a time: constant-property materials with the factor table
  c.pairs = (p->l3_pairs && !c.persist && p->src3tab && kconst && p->L3.nodes[2] >= 3) ? 1 : 0;
  // every later kernel of the call launches as a programmatic dependent of the one before it
  const gm::PdlScope pdl(p->pdl != 0);

  // Level-1 S1 from Level 2 at the overlap, substrate forced
  gm_restrict_s1_args s1;
  memset(&s1, 0, sizeof(s1));
  s1.dtype = p->dtype;
  for (int d = 0; d < 3; ++d) {
    s1.n[d] = p->r21.n[d];
    s1.cidx[d] = p->r21_idx[d];
  }
  s1.map = p->r21;
  s1.cnx = p->L1.nodes[0];
  s1.cny = p->L1.nodes[1];
  s1.fine_ph = p->L2.ph;
  s1.coarse_ph = p->L1.ph;
  s1.substrate = p->L1.substrate;
  GM_TRY(gm_restrict_s1(&s1, c.st));

  // Level-2 sources of all N2 steps (mean over each step's N3 rows), once
  const long long nrhs2 = (long long)p->rhs2_n[0] * p->rhs2_n[1] * p->rhs2_n[2];
  memzero(c, p->src2, nrhs2 * p->N2);
  source(c, p->c32, p->xq32, p->rows, p->N2 * p->N3, p->src2, p->rhs2_lo, p->rhs2_n, p->N2, nrhs2);

  // Level-1 right-hand side and predictor
  memzero(c, p->rhs1, nrhs1);
  source(c, p->c31, p->xq31, p->rows, p->N2 * p->N3, p->rhs1, p->rhs1_lo, p->rhs1_n);
  couple(c, p->c31, p->L3, p->rhs1, p->rhs1_lo, p->rhs1_n, p->L3.Tp, nullptr, nullptr, nullptr);
  couple(c, p->c21, p->L2, p->rhs1, p->rhs1_lo, p->rhs1_n, p->L2.Tp, nullptr, nullptr, nullptr);
  level(c, p->L1, p->L1_ne_planes, p->L1.T, p->T1p, p->dts, p->L1.ph, nullptr, p->rhs1, p->rhs1_lo, p->rhs1_n,
        nullptr, 1, nullptr, nullptr, nullptr, 0.0, nullptr, nullptr);

  // pass 1 (predictor)
  PassOut o = l2_pass(c, p->T1p, false);
  new_tprime(c, p->r21, p->r21_idx, p->L1, p->bc12, p->L2, o.T2, p->T1p, p->Tp2w, p->inj21);
  couple(c, p->c31, p->L3, p->rhs1, p->rhs1_lo, p->rhs1_n, nullptr, o.Tp3, p->L3.Tp, p->dts);
  couple(c, p->c21, p->L2, p->rhs1, p->rhs1_lo, p->rhs1_n, nullptr, p->Tp2w, p->L2.Tp, p->dts);
  level(c, p->L1, p->L1_ne_planes, p->L1.T, p->T1c, p->dts, p->L1.ph, nullptr, p->rhs1, p->rhs1_lo, p->rhs1_n,
        nullptr, 1, nullptr, nullptr, nullptr, 0.0, nullptr, nullptr);

  // pass 2 (corrector) and the new state
  o = l2_pass(c, p->T1c, true);
  copy(c, p->L3.T, o.T3, n3 * c.esz);
  copy(c, p->L3.ph, o.ph3, n3);
  copy(c, p->L3.Tp, o.Tp3, n3 * c.esz);
  copy(c, p->L2.T, o.T2, n2 * c.esz);
  copy(c, p->L2.ph, o.ph2, n2);
  new_tprime(c, p->r21, p->r21_idx, p->L1, p->bc12, p->L2, p->L2.T, p->T1c, p->L2.Tp, p->inj21);
  copy(c, p->L1.T, p->T1c, n1 * c.esz);

  // Level-0 S1 store at the Level-3 window
  gm_l0_args l0;
  memset(&l0, 0, sizeof(l0));
  for (int d = 0; d < 3; ++d) {
    l0.n[d] = p->L3.nodes[d];
    l0.idx[d] = p->l0_idx3[d];
  }
  l0.l0_nx = p->L0_nx;
  l0.l0_ny = p->L0_ny;
  l0.l0_bits = p->L0;
  l0.ph = p->L3.ph;
  GM_TRY(gm_l0_scatter(&l0, c.st));
  return c.rc;
}

// Graph mode: the call's launches are captured from the stream, applied to
// the executable graph of the previous call on this stream (same topology;
// only parameters change between calls), and launched as one graph.  The
// first call on a stream issues directly (it fills the launch-shape caches).
struct GraphSlot {
  void* stream = nullptr;
  cudaGraphExec_t exec = nullptr;
  int calls = 0;
};
thread_local GraphSlot g_slots[8];

GraphSlot* slot_for(void* stream) {
  for (auto& s : g_slots)
    if (s.calls > 0 && s.stream == stream) return &s;
  for (auto& s : g_slots)
    if (s.calls == 0) {
      s.stream = stream;
      return &s;
    }
  return nullptr;
}

int subcycle_graph(const gm_subcycle_plan* p, const gm_props* props, void* stream) {
  if (!stream) return subcycle_issue(p, props, stream);  // the legacy default stream cannot be captured
  GraphSlot* slot = slot_for(stream);
  if (!slot || slot->calls++ == 0) return subcycle_issue(p, props, stream);
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return GM_ERR_CUDA;
  const int rc = subcycle_issue(p, props, stream);
  cudaGraph_t graph = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(st, &graph);
  if (rc != GM_OK || ce != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    return rc != GM_OK ? rc : GM_ERR_CUDA;
  }
  int out = GM_OK;
  if (slot->exec) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(slot->exec, graph, &info) != cudaSuccess) {
      cudaGetLastError();  // clear the update failure; instantiate anew
      cudaGraphExecDestroy(slot->exec);
      slot->exec = nullptr;
    }
  }
  if (!slot->exec && cudaGraphInstantiate(&slot->exec, graph, 0) != cudaSuccess) out = GM_ERR_CUDA;
  if (out == GM_OK && cudaGraphLaunch(slot->exec, st) != cudaSuccess) out = GM_ERR_LAUNCH;
  cudaGraphDestroy(graph);
  return out;
}

}  // namespace

// ---------------------------------------------------------------------------
// Many instances: their subcycle calls as one CUDA graph of parallel branches.
// ---------------------------------------------------------------------------
namespace {

// Streams and events of the branches, created once per (calling thread,
// branch) and kept for the life of the process.
struct Branches {
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> joins;
  cudaEvent_t fork = nullptr;
  int ensure(int nb) {
    if (!fork && cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess) return GM_ERR_CUDA;
    while ((int)streams.size() < nb) {
      cudaStream_t s;
      cudaEvent_t e;
      if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return GM_ERR_CUDA;
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return GM_ERR_CUDA;
      streams.push_back(s);
      joins.push_back(e);
    }
    return GM_OK;
  }
};
thread_local Branches g_branches;

struct BatchSlot {
  void* stream = nullptr;
  int nb = 0;
  cudaGraphExec_t exec = nullptr;
  int calls = 0;
};
thread_local BatchSlot g_bslots[4];

// Issue the nb calls, instance i on branch stream i forked from `stream` and
// joined back into it (captured or not).
int issue_branches(const gm_subcycle_plan* plans, int nb, const gm_props* props, cudaStream_t st) {
  Branches& b = g_branches;
  if (cudaEventRecord(b.fork, st) != cudaSuccess) return GM_ERR_CUDA;
  int rc = GM_OK;
  for (int i = 0; i < nb && rc == GM_OK; ++i) {
    if (cudaStreamWaitEvent(b.streams[i], b.fork, 0) != cudaSuccess) return GM_ERR_CUDA;
    rc = subcycle_issue(&plans[i], &props[i], b.streams[i]);
    if (cudaEventRecord(b.joins[i], b.streams[i]) != cudaSuccess) return GM_ERR_CUDA;
    if (cudaStreamWaitEvent(st, b.joins[i], 0) != cudaSuccess) return GM_ERR_CUDA;
  }
  return rc;
}

}  // namespace

extern "C" int gm_subcycle_batched(const gm_subcycle_plan* plans, int nb, const gm_props* props, void* stream) {
  if (!plans || !props || nb < 1 || !stream) return GM_ERR_ARG;
  for (int i = 0; i < nb; ++i) {
    if (!plan_ok(&plans[i]) || (plans[i].dtype != GM_F32 && plans[i].dtype != GM_F64)) return GM_ERR_ARG;
    if (plans[i].persist) return GM_ERR_ARG;  // cooperative launches of concurrent branches are not co-scheduled
  }
  if (g_branches.ensure(nb) != GM_OK) return GM_ERR_CUDA;
  cudaStream_t st = (cudaStream_t)stream;
  BatchSlot* slot = nullptr;
  for (auto& sl : g_bslots)
    if (sl.calls > 0 && sl.stream == stream && sl.nb == nb) slot = &sl;
  if (!slot)
    for (auto& sl : g_bslots)
      if (sl.calls == 0) {
        sl.stream = stream;
        sl.nb = nb;
        slot = &sl;
        break;
      }
  // the first call of a batch issues directly (it fills the launch-shape caches)
  if (!slot || slot->calls++ == 0) return issue_branches(plans, nb, props, st);
  if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return GM_ERR_CUDA;
  const int rc = issue_branches(plans, nb, props, st);
  cudaGraph_t graph = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(st, &graph);
  if (rc != GM_OK || ce != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    return rc != GM_OK ? rc : GM_ERR_CUDA;
  }
  int out = GM_OK;
  if (slot->exec) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(slot->exec, graph, &info) != cudaSuccess) {
      cudaGetLastError();
      cudaGraphExecDestroy(slot->exec);
      slot->exec = nullptr;
    }
  }
  if (!slot->exec && cudaGraphInstantiate(&slot->exec, graph, 0) != cudaSuccess) out = GM_ERR_CUDA;
  if (out == GM_OK && cudaGraphLaunch(slot->exec, st) != cudaSuccess) out = GM_ERR_LAUNCH;
  cudaGraphDestroy(graph);
  return out;
}

extern "C" int gm_subcycle(const gm_subcycle_plan* p, const gm_props* props, void* stream) {
  if (!plan_ok(p) || !props || (p->dtype != GM_F32 && p->dtype != GM_F64)) return GM_ERR_ARG;
  return p->graph ? subcycle_graph(p, props, stream) : subcycle_issue(p, props, stream);
}
