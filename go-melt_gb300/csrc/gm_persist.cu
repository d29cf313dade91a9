// Level-3 fine steps of one Level-2 step in one launch (persistent kernel).
//
// The reference runs the N3 fine steps of a Level-2 step as a lax.scan of
// computeSolutions_L3 calls (go_melt/computeFunctions.py:3404-3430 and
// :3586-3622, each step :2960-3054 + the clamp and melt-time update).  Here
// one cooperative launch keeps the whole Level-3 window resident in shared
// memory for all N3 steps: CTA c owns a tile of node columns (tw x-columns x
// ty y-rows, all z planes) plus a one-column halo ring, in two shared-memory
// buffers (old / new step).  Between steps the CTAs exchange only their tile
// edges: each writes its edge columns to a full-size field in global memory
// (L2-resident), publishes the step with a release store of its flag, waits
// (acquire loads, bounded in time) for the flags of its up to eight
// neighbours and reads its halo ring back.  Two exchange fields alternate by
// step parity, so a CTA never overwrites edge values a neighbour may still be
// reading (it only writes step s+2 after every neighbour has published step
// s+1, which they did after reading step s).
//
// The per-node arithmetic is that of the one-step separable kernel
// (level_sep_kernel, bc_mode 3, laser factors from the step's table, melt
// time with the corrector's accumulators): same expressions in the same
// order, so both paths give the same bits.
//
// Failure handling: every wait gives up after about one second (clock64),
// sets bit GM_PERSIST_TIMEOUT of the status word and makes its CTA return;
// the CTAs waiting on it time out in turn, so the launch ends.  The final
// field is checked for non-finite values or values above 1e5 K (the
// reference driver's printLevelMaxMin bound): bit GM_PERSIST_BAD_T.
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <utility>

#include "gm_common.cuh"
#include "gm_sep.cuh"

namespace gm {

template <typename real>
struct PersistK {
  int nx, ny, nz, ntop;
  int tw, ty, txn, tyn, nseg;  // tile width (x columns), rows; tiles per axis; z segments per row
  int nsteps, nsub;
  unsigned base;
  int hold;  // 0, or 1 + a tile that withholds its counters (failure injection)
  long long substrate;
  const real* T_in;
  real* T_out;
  const uint8_t* ph_in;
  uint8_t* ph_out;
  real* xb0;
  real* xb1;
  unsigned* flags;
  int* status;
  const real* ringA;
  const real* ringB;
  const real* src_tab;
  const double* rows;
  real* accum;
  real* max_accum;
  Props<real> p;
  real sa1, sb1, sb2, smass, w2;
};

constexpr int PERSIST_MAX_THREADS = 768;
constexpr long long PERSIST_WAIT_CYCLES = 2000000000LL;  // about one second at the GB300's clocks

// Publish a counter: a release fence at GPU scope (it orders the CTA's
// writes, which the preceding barrier made this thread's) and the store.
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
  asm volatile("fence.acq_rel.gpu;\n st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Shared memory of a CTA: two T buffers [nz][ty + 2][32] (lane = x - X0,
// halo rows 0 and ty + 1), then the phase bytes of the owned nodes
// [nz][ty][32].
__host__ __device__ inline size_t persist_smem(int nz, int ty, size_t esz) {
  return 2 * (size_t)nz * (ty + 2) * 32 * esz + (size_t)nz * ty * 32;
}

template <typename real, bool ACC>
__global__ void __launch_bounds__(PERSIST_MAX_THREADS, 1) level3_persist_kernel(const PersistK<real> a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ int s_abort;
  constexpr unsigned FULL = 0xffffffffu;
  const int nx = a.nx, ny = a.ny, nz = a.nz, nxy = nx * ny, ntop = a.ntop;
  const int TY = a.ty, RYH = TY + 2, TW = a.tw;
  const int plane = RYH * 32;
  real* const B0 = (real*)smraw;
  real* const B1 = B0 + (size_t)nz * plane;
  uint8_t* const PH = (uint8_t*)(B1 + (size_t)nz * plane);
  const int tile = blockIdx.x;
  const int bx = tile % a.txn, by = tile / a.txn;
  const int X0 = bx * TW - 1, Y0 = by * TY - 1;  // coordinates of lane 0 and halo row 0
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int x = X0 + lane;
  const bool xin = x >= 0 && x < nx;
  const Props<real>& P = a.p;
  const int subs = a.substrate > (long long)nxy * nz ? nxy * nz : (int)a.substrate;

  // ---- the tile and its halo ring at the step start; phases of owned nodes ----
  for (int k = threadIdx.x; k < nz * plane; k += blockDim.x) {
    const int l = k & 31, i = (k >> 5) % RYH, z = k / plane;
    const int xx = X0 + l, yy = Y0 + i;
    B0[k] = (xx >= 0 && xx < nx && yy >= 0 && yy < ny) ? a.T_in[xx + yy * nx + z * nxy] : (real)0;
    B1[k] = (real)0;
  }
  for (int k = threadIdx.x; k < nz * TY * 32; k += blockDim.x) {
    const int l = k & 31, r = (k >> 5) % TY, z = k / (TY * 32);
    const int xx = X0 + l, yy = Y0 + 1 + r;
    PH[k] = (l >= 1 && l <= TW && xx < nx && yy < ny) ? a.ph_in[xx + yy * nx + z * nxy] : (uint8_t)0;
  }
  if (threadIdx.x == 0) s_abort = 0;
  __syncthreads();

  // ---- this warp's task: tile row r, z segment seg of the interior planes ----
  const int r = warp / a.nseg, seg = warp % a.nseg;
  const int y = Y0 + 1 + r;
  const bool own = lane >= 1 && lane <= TW && xin && y < ny;  // the lane's node column belongs to the tile
  const bool dir = x == 0 || x == nx - 1 || y == 0 || y == ny - 1;  // Dirichlet column
  // interior planes 1 .. ntop-1 split over the segments, the top plane
  // (surface flux) counted as two planes of work of the last segment
  const int nint = ntop - 1, units = nint + 2;
  const int za = 1 + (seg * units) / a.nseg;
  const int zb = seg == a.nseg - 1 ? ntop : 1 + ((seg + 1) * units) / a.nseg;
  const bool top_task = seg == a.nseg - 1, bottom_task = seg == 0;
  const real a1 = a.sa1, b1 = a.sb1, b2 = a.sb2;
  const int L = nx + ny + nz;
  const int col = x + y * nx;  // node id of plane 0 in this column (used only when own)

  for (int s = 0; s < a.nsteps; ++s) {
    const real* cur = (s & 1) ? B1 : B0;
    real* nxt = (s & 1) ? B0 : B1;
    const real dt = (real)a.rows[7LL * s + 5];
    const real minv = dt / a.smass;
    const double al = (double)(s + 1) / (double)a.nsub;
    const real alpha = (real)al, beta = (real)(1.0 - al);
    const real* tb = a.src_tab + (size_t)s * L;
    const real sx = xin ? tb[x] : (real)0;
    const real sxy = rmul(sx, (y < ny) ? tb[nx + y] : (real)0);

    // step s+1 lives in exchange field (s+1) & 1; the last step publishes nothing
    real* const xbn = s == a.nsteps - 1 ? nullptr : ((s & 1) ? a.xb0 : a.xb1);
    const bool edge = lane == 1 || lane == TW || r == 0 || r == TY - 1;  // read by a neighbouring tile
    // new phase, value and melt time of the owned node at plane p; edge
    // nodes also go to the exchange field at once
    auto finish = [&](int p, real Tn, real Told) {
      Tn = fmax(Tn, P.T_amb);
      nxt[(p * RYH + r + 1) * 32 + lane] = Tn;
      const int id = col + p * nxy;
      if (edge && xbn) __stcg(&xbn[id], Tn);
      uint8_t& phr = PH[(p * TY + r) * 32 + lane];
      const uint32_t ph = phr;
      const bool s2 = Told >= P.T_liquidus;
      const bool s1 = (ph & PH_S1) || s2 || id < subs;
      phr = (uint8_t)((s1 ? PH_S1 : 0u) | (s2 ? PH_S2 : 0u));
      if (ACC && s2) {
        const real cAcc = a.accum[id], cMacc = a.max_accum[id];
        const bool prev2 = (ph & PH_S2) != 0;
        const real racc = prev2 ? (real)0 : cAcc;
        a.max_accum[id] = fmax(racc, cMacc);
        a.accum[id] = rsub(radd(cAcc, dt), racc);
      }
    };
    auto ring_value = [&](int p) {
      const int id = col + p * nxy;
      return rfma(alpha, a.ringA[id], rmul(beta, a.ringB[id]));
    };
    auto at = [&](const real* b, int p, int i) { return b[(p * RYH + i) * 32 + lane]; };

    // the step's z source factors of this warp's planes za .. za+31, one a lane
    const real szl = (za + lane <= ntop) ? tb[nx + ny + za + lane] : (real)0;
    // interior planes [za, zb): rows r .. r+2 of the halo-indexed buffer,
    // walked with pointers (plane stride `plane` values)
    if (za < zb) {
      const real* c = cur + (size_t)(za - 1) * plane + r * 32 + lane;
      real Tm0 = c[0], Tm1 = c[32], Tm2 = c[64];
      c += plane;
      real T00 = c[0], T01 = c[32], T02 = c[64];
      for (int p = za; p < zb; ++p) {
        c += plane;
        const real Tp0 = c[0], Tp1 = c[32], Tp2 = c[64];
        const real s0 = radd(Tm0, Tp0), s1 = radd(Tm1, Tp1), s2 = radd(Tm2, Tp2);
        const real Zm0 = rfma((real)4, T00, s0), Zm1 = rfma((real)4, T01, s1), Zm2 = rfma((real)4, T02, s2);
        const real Zk0 = rfma((real)2, T00, -s0), Zk1 = rfma((real)2, T01, -s1), Zk2 = rfma((real)2, T02, -s2);
        const real u = radd(Zm0, Zm2);
        const real w = radd(Zk0, Zk2);
        const real A = rmul(a1, rfma((real)4, Zm1, u));
        const real B = rfma(b1, rfma((real)2, Zm1, -u), rmul(b2, rfma((real)4, Zk1, w)));
        const real D = rsub(B, A);
        const real Dl = __shfl_up_sync(FULL, D, 1), Dr = __shfl_down_sync(FULL, D, 1);
        const real sz = __shfl_sync(FULL, szl, p - za);
        if (own) {
          const real Told = T01;
          real Tn;
          if (dir) {
            Tn = ring_value(p);
          } else {
            const real KT = radd(rfma((real)2, A, rmul((real)4, B)), radd(Dl, Dr));
            const real Rt = rfma(sxy, sz, -KT);
            Tn = rfma(Rt, minv, Told);
          }
          finish(p, Tn, Told);
        }
        Tm0 = T00;
        Tm1 = T01;
        Tm2 = T02;
        T00 = Tp0;
        T01 = Tp1;
        T02 = Tp2;
      }
    }
    // top plane ntop: one-sided z operators, lumped mass of 4 elements, surface flux
    if (top_task) {
      RegCol<real, 3> t0c;
      real Tm[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        Tm[i] = at(cur, ntop - 1, r + i);
        t0c.v[i] = at(cur, ntop, r + i);
      }
      const RegCol<real, 1> sf = sep_surface<real, 1>(P, a.w2, x, nx, y, ny, t0c);
      const real szt = __shfl_sync(FULL, szl, ntop - za);
      real Zm[3], Zk[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        Zm[i] = rfma((real)2, t0c.v[i], Tm[i]);
        Zk[i] = rsub(t0c.v[i], Tm[i]);
      }
      const real u = radd(Zm[0], Zm[2]);
      const real w = radd(Zk[0], Zk[2]);
      const real A = rmul(a1, rfma((real)4, Zm[1], u));
      const real B = rfma(b1, rfma((real)2, Zm[1], -u), rmul(b2, rfma((real)4, Zk[1], w)));
      const real D = rsub(B, A);
      const real Dl = __shfl_up_sync(FULL, D, 1), Dr = __shfl_down_sync(FULL, D, 1);
      if (own) {
        const real Told = t0c.v[1];
        real Tn;
        if (dir) {
          Tn = ring_value(ntop);
        } else {
          const real KT = radd(rfma((real)2, A, rmul((real)4, B)), radd(Dl, Dr));
          const real Rt = radd(rfma(sxy, szt, -KT), sf.v[0]);
          Tn = rfma(Rt, (real)2 * minv, Told);
        }
        finish(ntop, Tn, Told);
      }
    }
    // bottom plane: Dirichlet
    if (bottom_task && own) finish(0, ring_value(0), at(cur, 0, r + 1));
    __syncthreads();

    if (s == a.nsteps - 1) break;

    // ---- publish step s+1: every edge node was written to the exchange field above ----
    const real* xb = xbn;
    const unsigned target = a.base + (unsigned)(s + 1);
    if (threadIdx.x == 0 && tile + 1 != a.hold) st_release(a.flags + tile, target);
    // ---- wait for the neighbours' step s+1 (bounded) ----
    if (threadIdx.x < 9 && threadIdx.x != 4) {
      const int nbx = bx + (int)(threadIdx.x % 3) - 1, nby = by + (int)(threadIdx.x / 3) - 1;
      if (nbx >= 0 && nbx < a.txn && nby >= 0 && nby < a.tyn) {
        const unsigned* f = a.flags + (nbx + nby * a.txn);
        const long long t0 = clock64();
        while ((int)(ld_acquire(f) - target) < 0) {
          if (clock64() - t0 > PERSIST_WAIT_CYCLES) {
            s_abort = 1;
            atomicOr(a.status, GM_PERSIST_TIMEOUT);
            break;
          }
        }
      }
    }
    __syncthreads();
    if (s_abort) return;
    // ---- halo ring of step s+1 from the neighbours' edges ----
    const int H = 2 * RYH + 2 * TW;
    for (int k = threadIdx.x; k < nz * H; k += blockDim.x) {
      const int z = k / H, e = k - z * H;
      int i, l;
      if (e < RYH) {
        i = e;
        l = 0;
      } else if (e < 2 * RYH) {
        i = e - RYH;
        l = TW + 1;
      } else if (e < 2 * RYH + TW) {
        i = 0;
        l = 1 + e - 2 * RYH;
      } else {
        i = RYH - 1;
        l = 1 + e - 2 * RYH - TW;
      }
      const int xx = X0 + l, yy = Y0 + i;
      if (xx >= 0 && xx < nx && yy >= 0 && yy < ny) nxt[(z * RYH + i) * 32 + l] = __ldcg(&xb[xx + yy * nx + z * nxy]);
    }
    __syncthreads();
  }

  // ---- the window after the last step: owned nodes and phases ----
  const real* fin = (a.nsteps & 1) ? B1 : B0;
  bool bad = false;
  for (int k = threadIdx.x; k < nz * TY * 32; k += blockDim.x) {
    const int l = k & 31, rr = (k >> 5) % TY, z = k / (TY * 32);
    const int xx = X0 + l, yy = Y0 + 1 + rr;
    if (l >= 1 && l <= TW && xx < nx && yy < ny) {
      const int id = xx + yy * nx + z * nxy;
      const real v = fin[(z * RYH + rr + 1) * 32 + l];
      a.T_out[id] = v;
      a.ph_out[id] = PH[k];
      bad = bad || !(v <= (real)1e5);  // also true for NaN
    }
  }
  if (__any_sync(FULL, bad) && lane == 0) atomicOr(a.status, GM_PERSIST_BAD_T);
  // every flag of a completed launch ends at base + nsteps (the next launch's base)
  __syncthreads();
  if (threadIdx.x == 0 && tile + 1 != a.hold) st_release(a.flags + tile, a.base + (unsigned)a.nsteps);
}

}  // namespace gm

using namespace gm;

namespace {

struct PersistShape {
  int tw, ty, txn, tyn, nseg, threads;
  size_t smem;
};

int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    n = v > 0 ? v : 152;
  }
  return n;
}

// Dynamic shared memory a CTA may use: the device's opt-in maximum less a
// margin for the kernel's static shared memory.
size_t smem_cap() {
  static size_t cap = 0;
  if (cap == 0) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cap = (v > 1024 ? (size_t)v : 232448) - 256;
  }
  return cap;
}

// Tiles: x-tiles of at most 30 output columns (one warp with its two halo
// lanes), balanced (tw = ceil(nx / txn)); rows ty, the smallest number that
// gives one tile per SM at most; z segments so that a CTA has up to 24 warps
// and a segment at least 4 planes.
bool persist_shape(int nx, int ny, int nz, size_t esz, PersistShape* s) {
  if (nx < 3 || ny < 3 || nz < 3) return false;
  const int sms = sm_count();
  s->txn = cdiv(nx, 30);
  s->tw = cdiv(nx, s->txn);
  if ((s->txn - 1) * s->tw >= nx) return false;  // every x-tile holds at least one column
  const int per_col = sms / s->txn;
  if (per_col < 1) return false;
  s->ty = cdiv(ny, per_col);
  s->tyn = cdiv(ny, s->ty);
  const int seg_cap = PERSIST_MAX_THREADS / 32 / s->ty;
  if (seg_cap < 1) return false;
  const int nint = nz - 2;
  int nseg = cdiv(nint, 4);
  if (nseg > seg_cap) nseg = seg_cap;
  if (nseg < 1) nseg = 1;
  s->nseg = nseg;
  if ((nint + 2) / nseg + 3 > 32) return false;  // a segment's planes, top included, one z factor a lane
  s->threads = 32 * s->ty * nseg;
  s->smem = persist_smem(nz, s->ty, esz);
  return s->smem <= smem_cap();
}

template <typename real, bool ACC>
cudaError_t persist_attr() {
  static std::once_flag once;
  static cudaError_t err = cudaSuccess;
  std::call_once(once, [] {
    err = cudaFuncSetAttribute(level3_persist_kernel<real, ACC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem_cap());
  });
  return err;
}

// Whether every tile of shape s can be resident at once (cooperative launch).
// The occupancy of each (threads, shared memory) is queried once and cached,
// so calls made during a stream capture repeat no device query.
template <typename real, bool ACC>
bool persist_resident(const PersistShape& s) {
  static std::mutex mu;
  static std::map<std::pair<int, size_t>, int> occ_of;
  if (persist_attr<real, ACC>() != cudaSuccess) return false;
  int occ = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = occ_of.find({s.threads, s.smem});
    if (it != occ_of.end()) {
      occ = it->second;
    } else {
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, level3_persist_kernel<real, ACC>, s.threads,
                                                        s.smem) != cudaSuccess) {
        cudaGetLastError();
        occ = 0;
      }
      occ_of[{s.threads, s.smem}] = occ;
    }
  }
  return (long long)occ * sm_count() >= (long long)s.txn * s.tyn;
}

// The shape of a window for a dtype, if both variants (with and without melt
// time) fit on the device.
bool persist_ok(int dtype, const int nodes[3], PersistShape* s) {
  const size_t esz = dtype == GM_F64 ? 8 : 4;
  if (!persist_shape(nodes[0], nodes[1], nodes[2], esz, s)) return false;
  return dtype == GM_F64 ? persist_resident<double, false>(*s) && persist_resident<double, true>(*s)
                         : persist_resident<float, false>(*s) && persist_resident<float, true>(*s);
}

template <typename real, bool ACC>
int launch_persist(const PersistK<real>& a, const PersistShape& s, cudaStream_t st) {
  if (!persist_resident<real, ACC>(s)) return GM_ERR_UNSUPPORTED;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(s.txn * s.tyn);
  cfg.blockDim = dim3(s.threads);
  cfg.dynamicSmemBytes = s.smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;  // every CTA resident at once: the waits cannot starve
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, level3_persist_kernel<real, ACC>, a) != cudaSuccess) return GM_ERR_LAUNCH;
  return GM_OK;
}

bool props_constant(const gm_props* p) {
  return p->k_powder == p->k_bulk_a0 && p->k_fluid == p->k_bulk_a0 && p->k_bulk_a1 == 0.0 &&
         p->cp_solid_a1 == 0.0 && p->cp_mushy == p->cp_solid_a0 && p->cp_fluid == p->cp_solid_a0;
}

template <typename real>
int do_persist(const gm_persist_args* g, const gm_props* pr, const PersistShape& s, cudaStream_t st) {
  PersistK<real> a;
  a.nx = g->nodes[0];
  a.ny = g->nodes[1];
  a.nz = g->nodes[2];
  a.ntop = a.nz - 1;
  a.tw = s.tw;
  a.ty = s.ty;
  a.txn = s.txn;
  a.tyn = s.tyn;
  a.nseg = s.nseg;
  a.nsteps = g->nsteps;
  a.nsub = g->nsub;
  a.base = g->base;
  a.hold = g->hold;
  a.substrate = g->substrate;
  a.T_in = (const real*)g->T_in;
  a.T_out = (real*)g->T_out;
  a.ph_in = g->ph_in;
  a.ph_out = g->ph_out;
  a.xb0 = (real*)g->xbuf[0];
  a.xb1 = (real*)g->xbuf[1];
  a.flags = g->flags;
  a.status = g->status;
  a.ringA = (const real*)g->ring_new;
  a.ringB = (const real*)g->ring_old;
  a.src_tab = (const real*)g->src_tab;
  a.rows = g->rows;
  a.accum = (real*)g->accum;
  a.max_accum = (real*)g->max_accum;
  a.p = make_props<real>(*pr);
  // the separable constants of the one-step kernel (make_levelk), formed in double
  const double hx = g->h[0], hy = g->h[1], hz = g->h[2];
  const double kc = pr->k_fluid / 1000.0;
  a.sa1 = (real)(kc * hy * hz / (36.0 * hx));
  a.sb1 = (real)(kc * hx * hz / (36.0 * hy));
  a.sb2 = (real)(kc * hx * hy / (36.0 * hz));
  a.smass = (real)(hx * hy * hz * pr->rho * pr->cp_fluid);
  a.w2 = (real)(hx * hy / 4.0);
  return g->accum ? launch_persist<real, true>(a, s, st) : launch_persist<real, false>(a, s, st);
}

}  // namespace

extern "C" long long gm_level3_persist_flags(const int nodes[3]) {
  PersistShape s;
  if (!nodes || !persist_shape(nodes[0], nodes[1], nodes[2], 4, &s)) return -1;
  return (long long)s.txn * s.tyn;
}

extern "C" int gm_level3_persist_shape(int dtype, const int nodes[3], int out[4]) {
  if (!nodes || !out || (dtype != GM_F32 && dtype != GM_F64)) return GM_ERR_ARG;
  PersistShape s;
  if (!persist_ok(dtype, nodes, &s)) return GM_ERR_UNSUPPORTED;
  out[0] = s.txn * s.tyn;
  out[1] = s.tw;
  out[2] = s.ty;
  out[3] = s.nseg;
  return GM_OK;
}

extern "C" int gm_level3_persist(const gm_persist_args* g, const gm_props* p, void* stream) {
  if (!g || !p || (g->dtype != GM_F32 && g->dtype != GM_F64)) return GM_ERR_ARG;
  if (!g->T_in || !g->T_out || !g->ph_in || !g->ph_out || !g->ring_new || !g->ring_old || !g->src_tab ||
      !g->rows || !g->xbuf[0] || !g->xbuf[1] || !g->flags || !g->status)
    return GM_ERR_ARG;
  if (g->nsteps < 1 || g->nsub < 1 || (g->accum == nullptr) != (g->max_accum == nullptr) || g->hold < 0)
    return GM_ERR_ARG;
  if (g->T_in == g->xbuf[0] || g->T_in == g->xbuf[1] || g->xbuf[0] == g->xbuf[1] || g->T_in == g->T_out ||
      (const void*)g->ph_in == (const void*)g->ph_out)
    return GM_ERR_ARG;
  if ((long long)g->nodes[0] * g->nodes[1] * g->nodes[2] >= (1LL << 31)) return GM_ERR_TOO_LARGE;
  if (!props_constant(p)) return GM_ERR_UNSUPPORTED;
  PersistShape s;
  if (!persist_ok(g->dtype, g->nodes, &s)) return GM_ERR_UNSUPPORTED;
  if (g->flags_cap < (long long)s.txn * s.tyn) return GM_ERR_TOO_LARGE;
  if (g->hold > s.txn * s.tyn) return GM_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  return g->dtype == GM_F32 ? do_persist<float>(g, p, s, st) : do_persist<double>(g, p, s, st);
}
