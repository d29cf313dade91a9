// Inter-level transfer kernels: prolongation (gather), restriction + T',
// Level-1 S1 restriction and the Level-0 phase store gather/scatter.
//
// All maps are separable: a target point (i,j,k) of a tensor grid of points is
// located in the source grid by three per-axis tables (gm_map3), so no kernel
// stores or reads an 8-weight-per-point matrix.
#include "gm_common.cuh"

namespace gm {

template <typename real>
struct InterpK {
  int n[3];
  int nterms;
  Map3<real> map[3];
  const real* src[3];
  real coef[3];
  const real* base;
  real* out;
  real* out_term;
  int which_term;
};

// out[t] = base[t] + sum_k coef_k * I_k(src_k)[t]; optionally out_term = I_which.
// interpolatePoints / interpolate_w_matrix (computeFunctions.py:1110-1210),
// the T' of getNewTprime (:2097) and the field remap of moveEverything
// (:2427-2459).
// Launch: x threads over i, grid (ceil(n0 / blockDim.x), ceil(n1 / IROWS),
// n2): no index is divided, and a thread keeps its x weights over IROWS rows.
// The eight trilinear weights and their validity rule are those of
// map3_weights.
constexpr int IROWS = 8;
template <typename real>
__global__ void interp_kernel(const InterpK<real> a) {
  pdl_begin();
  const int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.z;
  if (i >= a.n[0]) return;
  int ex[3], ez[3];
  real x0[3], x1[3], z0[3], z1[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    if (q >= a.nterms) break;
    const Map3<real>& m = a.map[q];
    ex[q] = m.ax[0].e[i];
    x0[q] = m.ax[0].w[2 * i];
    x1[q] = m.ax[0].w[2 * i + 1];
    ez[q] = m.ax[2].e[k];
    z0[q] = m.ax[2].w[2 * k];
    z1[q] = m.ax[2].w[2 * k + 1];
  }
  const int j1 = min(a.n[1], (int)(blockIdx.y + 1) * IROWS);
  for (int j = blockIdx.y * IROWS; j < j1; ++j) {
    const long long t = i + (long long)a.n[0] * (j + (long long)a.n[1] * k);
    real acc = a.base ? a.base[t] : (real)0;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      if (q >= a.nterms) break;
      const Map3<real>& m = a.map[q];
      const int ey = m.ax[1].e[j];
      const real y0 = m.ax[1].w[2 * j], y1 = m.ax[1].w[2 * j + 1];
      real w8[8];
      w8[0] = x0[q] * y0 * z0[q];
      w8[1] = x1[q] * y0 * z0[q];
      w8[2] = x1[q] * y1 * z0[q];
      w8[3] = x0[q] * y1 * z0[q];
      w8[4] = x0[q] * y0 * z1[q];
      w8[5] = x1[q] * y0 * z1[q];
      w8[6] = x1[q] * y1 * z1[q];
      w8[7] = x0[q] * y1 * z1[q];
      bool ok = true;
#pragma unroll
      for (int r = 0; r < 8; ++r) ok = ok && (w8[r] >= (real)-1e-2) && (w8[r] <= (real)(1 + 1e-2));
#pragma unroll
      for (int r = 0; r < 8; ++r) w8[r] = ok ? fmin(fmax(w8[r], (real)0), (real)1) : (real)0;
      const int sx = 1, sy = m.src_nx, sz = m.src_nx * m.src_ny;
      const int b = ex[q] + ey * sy + ez[q] * sz;
      const real* u = a.src[q];
      const real v = w8[0] * u[b] + w8[1] * u[b + sx] + w8[2] * u[b + sx + sy] + w8[3] * u[b + sy] +
                     w8[4] * u[b + sz] + w8[5] * u[b + sx + sz] + w8[6] * u[b + sx + sy + sz] +
                     w8[7] * u[b + sy + sz];
      if (a.out_term && q == a.which_term) a.out_term[t] = v;
      acc = acc + a.coef[q] * v;
    }
    a.out[t] = acc;
  }
}

// Materialised weights (interpolatePointsMatrix, :1028-1107).
template <typename real>
__global__ void interp_matrix_kernel(const Map3<real> m, int n0, int n1, int n2, real* Nc, int* node) {
  const long long tot = (long long)n0 * n1 * n2;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % n0), j = (int)((t / n0) % n1), k = (int)(t / ((long long)n0 * n1));
    real w8[8];
    const int b = map3_weights(m, i, j, k, w8);
    const int sx = 1, sy = m.src_nx, sz = m.src_nx * m.src_ny;
    const int off[8] = {0, sx, sx + sy, sy, sz, sx + sz, sx + sy + sz, sy + sz};
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      Nc[t * 8 + q] = w8[q];
      node[t * 8 + q] = b + off[q];
    }
  }
}

// interpolate_w_matrix (:1110-1128) with stored weights.
template <typename real>
__global__ void w_matrix_kernel(const real* Nc, const int* node, const real* T, real* out, long long n) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    real s = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) s += Nc[t * 8 + q] * T[node[t * 8 + q]];
    out[t] = s;
  }
}

// Restriction (getNewTprime, :2085-2093): coarse[idx] = fine field evaluated at
// the coordinates of the coarse nodes inside the fine window.
template <typename real>
__global__ void restrict_kernel(int n0, int n1, int n2, const Map3<real> m, const int* cx, const int* cy, const int* cz,
                                int cnx, int cny, const real* fine, real* coarse) {
  pdl_begin();
  const int tot = n0 * n1 * n2;  // < 2^31 (checked by the caller)
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += gridDim.x * blockDim.x) {
    const int i = t % n0, j = (t / n0) % n1, k = t / (n0 * n1);
    const real v = map3_apply(m, i, j, k, fine);
    coarse[cx[i] + (long long)cy[j] * cnx + (long long)cz[k] * cnx * cny] = v;
  }
}

// Restriction and T' in one pass (gm_tprime_inject): the prolongation of
// interp_kernel with the eight corner values taken from the fine field at
// coarse overlap nodes (their restricted value when the restriction is an
// injection), and the coarse overlap nodes written with those fine values.
// Reads of the coarse field touch only nodes outside the overlap, which no
// thread writes.  Per fine index and axis, cf0 / cf1 give the fine node
// coinciding with the low / high corner of its coarse element (-1: not an
// overlap index), so each corner value is one load after the tables.
constexpr int TROWS = 2;  // fine rows a thread
template <typename real>
struct TprimeK {
  int n[3];
  Map3<real> cmap;
  const int* cf0[3];
  const int* cf1[3];
  const int* c_of_f[3];
  int cnx, cny;
  const real* fine;
  real* coarse;
  real* out;
};

template <typename real>
__global__ void tprime_inject_kernel(const TprimeK<real> a) {
  pdl_begin();
  const int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.z;
  if (i >= a.n[0]) return;
  const Map3<real>& m = a.cmap;
  const int ex = m.ax[0].e[i], ez = m.ax[2].e[k];
  const real x0 = m.ax[0].w[2 * i], x1 = m.ax[0].w[2 * i + 1];
  const real z0 = m.ax[2].w[2 * k], z1 = m.ax[2].w[2 * k + 1];
  const int fx[2] = {a.cf0[0][i], a.cf1[0][i]};
  const int fz[2] = {a.cf0[2][k], a.cf1[2][k]};
  const int cfx = a.c_of_f[0][i], cfz = a.c_of_f[2][k];
  const long long fnxy = (long long)a.n[0] * a.n[1];
  const long long cnxy = (long long)a.cnx * a.cny;
  const int jb = blockIdx.y * TROWS;
  // the rows' tables first (independent loads), then the corner values
  int ey[TROWS], fy0[TROWS], fy1[TROWS], cfy[TROWS];
  real y0[TROWS], y1[TROWS];
#pragma unroll
  for (int r = 0; r < TROWS; ++r) {
    const int j = min(jb + r, a.n[1] - 1);
    ey[r] = m.ax[1].e[j];
    y0[r] = m.ax[1].w[2 * j];
    y1[r] = m.ax[1].w[2 * j + 1];
    fy0[r] = a.cf0[1][j];
    fy1[r] = a.cf1[1][j];
    cfy[r] = a.c_of_f[1][j];
  }
  constexpr int OX[8] = {0, 1, 1, 0, 0, 1, 1, 0}, OY[8] = {0, 0, 1, 1, 0, 0, 1, 1}, OZ[8] = {0, 0, 0, 0, 1, 1, 1, 1};
#pragma unroll
  for (int r = 0; r < TROWS; ++r) {
    const int j = jb + r;
    if (j >= a.n[1]) break;
    const long long t = i + (long long)a.n[0] * j + fnxy * k;
    real w8[8];
    w8[0] = x0 * y0[r] * z0;
    w8[1] = x1 * y0[r] * z0;
    w8[2] = x1 * y1[r] * z0;
    w8[3] = x0 * y1[r] * z0;
    w8[4] = x0 * y0[r] * z1;
    w8[5] = x1 * y0[r] * z1;
    w8[6] = x1 * y1[r] * z1;
    w8[7] = x0 * y1[r] * z1;
    bool ok = true;
#pragma unroll
    for (int q = 0; q < 8; ++q) ok = ok && (w8[q] >= (real)-1e-2) && (w8[q] <= (real)(1 + 1e-2));
#pragma unroll
    for (int q = 0; q < 8; ++q) w8[q] = ok ? fmin(fmax(w8[q], (real)0), (real)1) : (real)0;
    const int fy[2] = {fy0[r], fy1[r]};
    real u[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int gx = fx[OX[q]], gy = fy[OY[q]], gz = fz[OZ[q]];
      u[q] = (gx >= 0 && gy >= 0 && gz >= 0)
                 ? a.fine[gx + (long long)a.n[0] * gy + fnxy * gz]
                 : a.coarse[(ex + OX[q]) + (long long)a.cnx * (ey[r] + OY[q]) + cnxy * (ez + OZ[q])];
    }
    const real v = w8[0] * u[0] + w8[1] * u[1] + w8[2] * u[2] + w8[3] * u[3] + w8[4] * u[4] + w8[5] * u[5] +
                   w8[6] * u[6] + w8[7] * u[7];
    const real f = a.fine[t];
    a.out[t] = f + (real)-1 * v;
    if (cfx >= 0 && cfy[r] >= 0 && cfz >= 0) a.coarse[cfx + (long long)a.cnx * cfy[r] + cnxy * cfz] = f;
  }
}

// Level-1 S1 from Level 2 (subcycleGOMELT :3272-3278, updateStateProperties
// :2547-2556): interpolate the 0/1 S1 of Level 2 at the Level-1 overlap nodes;
// the stored bit is the value's use in computeStateProperties (S1 > 0.499),
// then the substrate override.
template <typename real>
__global__ void restrict_s1_kernel(int n0, int n1, int n2, const Map3<real> m, const int* cx, const int* cy,
                                   const int* cz, int cnx, int cny, const uint8_t* fine_ph, int fnx, int fny,
                                   uint8_t* coarse_ph, long long substrate) {
  pdl_begin();
  const long long tot = (long long)n0 * n1 * n2;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % n0), j = (int)((t / n0) % n1), k = (int)(t / ((long long)n0 * n1));
    real w8[8];
    const int b = map3_weights(m, i, j, k, w8);
    const int sx = 1, sy = fnx, sz = fnx * fny;
    const int off[8] = {0, sx, sx + sy, sy, sz, sx + sz, sx + sy + sz, sy + sz};
    real v = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) v += w8[q] * (real)(fine_ph[b + off[q]] & PH_S1);
    const long long id = cx[i] + (long long)cy[j] * cnx + (long long)cz[k] * cnx * cny;
    const bool s1 = (v > (real)0.499) || id < substrate;
    coarse_ph[id] = (uint8_t)((coarse_ph[id] & ~PH_S1) | (s1 ? PH_S1 : 0));
  }
  // S1[:substrate] = 1 on the whole level.  Overlap nodes below `substrate`
  // get the same byte from both loops (S1 set, S2 kept), so the order of the
  // two writes does not matter.
  for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < substrate;
       id += (long long)gridDim.x * blockDim.x)
    coarse_ph[id] |= PH_S1;
}

// Level-0 S1 store: one bit per node in 32-bit words, each (y, z) row of
// l0_nx nodes padded to whole words: node (x, y, z) is bit x % 32 of word
// (z * l0_ny + y) * l0_words_per_row(l0_nx) + x / 32.
__host__ __device__ inline long long l0_words_per_row(long long lnx) { return (lnx + 31) / 32; }

// Level-0 gather (moveEverything :2500-2502): window phase from the Level-0
// S1 store; S2 from the previous window's phase where the windows overlap
// (Level 0 holds S2 only inside the last scattered window, :2390-2392).
__global__ void l0_gather_kernel(int n0, int n1, int n2, const int* ix, const int* iy, const int* iz, long long lnx,
                                 long long lny, const uint32_t* l0, uint8_t* ph, const uint8_t* prev_ph, int plo0,
                                 int plo1, int plo2, int pn0, int pn1, int pn2) {
  const long long tot = (long long)n0 * n1 * n2;
  const long long wpr = l0_words_per_row(lnx);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % n0), j = (int)((t / n0) % n1), k = (int)(t / ((long long)n0 * n1));
    const int x = ix[i];
    const uint32_t w = l0[(iz[k] * lny + iy[j]) * wpr + (x >> 5)];
    uint8_t p = ((w >> (x & 31)) & 1u) ? PH_S1 : 0;
    if (prev_ph) {
      const int a = ix[i] - plo0, b = iy[j] - plo1, c = iz[k] - plo2;
      if (a >= 0 && a < pn0 && b >= 0 && b < pn1 && c >= 0 && c < pn2)
        p |= prev_ph[a + (long long)b * pn0 + (long long)c * pn0 * pn1] & PH_S2;
    }
    ph[t] = p;
  }
}

// Level-0 scatter (subcycleGOMELT :3628-3630): store the window's S1.  A bit
// that already holds the value is left alone; the others are set or cleared
// with an atomic on their word (neighbouring nodes share words).
__global__ void l0_scatter_kernel(int n0, int n1, int n2, const int* ix, const int* iy, const int* iz, long long lnx,
                                  long long lny, uint32_t* l0, const uint8_t* ph) {
  const long long tot = (long long)n0 * n1 * n2;
  const long long wpr = l0_words_per_row(lnx);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % n0), j = (int)((t / n0) % n1), k = (int)(t / ((long long)n0 * n1));
    const int x = ix[i];
    uint32_t* w = l0 + (iz[k] * lny + iy[j]) * wpr + (x >> 5);
    const uint32_t bit = 1u << (x & 31);
    const bool s1 = (ph[t] & PH_S1) != 0;
    const bool cur = (*w & bit) != 0;
    if (s1 && !cur) atomicOr(w, bit);
    if (!s1 && cur) atomicAnd(w, ~bit);
  }
}

// Node range [first, last) of the store set to `value` (whole words where the
// range covers them, atomics on the partial words at its ends per row).
__global__ void l0_fill_kernel(long long lnx, long long lny, long long lnz, long long first, long long last,
                               uint32_t* l0, int value) {
  const long long wpr = l0_words_per_row(lnx);
  const long long words = wpr * lny * lnz;
  for (long long wi = blockIdx.x * (long long)blockDim.x + threadIdx.x; wi < words;
       wi += (long long)gridDim.x * blockDim.x) {
    const long long row = wi / wpr, x0 = (wi - row * wpr) * 32;
    const long long id0 = row * lnx + x0;  // node id of bit 0 of this word
    uint32_t mask = 0;
    for (int b = 0; b < 32; ++b) {
      const long long id = id0 + b;
      if (x0 + b < lnx && id >= first && id < last) mask |= 1u << b;
    }
    if (mask == 0xffffffffu)
      l0[wi] = value ? 0xffffffffu : 0u;
    else if (mask)
      value ? atomicOr(l0 + wi, mask) : atomicAnd(l0 + wi, ~mask);
  }
}

inline int grid_for(long long n, int block = 256) {
  long long g = (n + block - 1) / block;
  if (g > 152 * 32) g = 152 * 32;
  return g < 1 ? 1 : (int)g;
}

template <typename real>
static int do_interp(const gm_interp_args* g, cudaStream_t st) {
  InterpK<real> a;
  for (int d = 0; d < 3; ++d) a.n[d] = g->n[d];
  a.nterms = g->nterms;
  for (int q = 0; q < 3; ++q) {
    if (q < g->nterms) {
      a.map[q] = make_map3<real>(g->map[q]);
      a.src[q] = (const real*)g->src[q];
      a.coef[q] = (real)g->coef[q];
    } else {
      a.src[q] = nullptr;
      a.coef[q] = 0;
    }
  }
  a.base = (const real*)g->base;
  a.out = (real*)g->out;
  a.out_term = (real*)g->out_term;
  a.which_term = g->which_term;
  const int bx = a.n[0] <= 256 ? 32 * cdiv(a.n[0], 32) : 256;
  launch_k(interp_kernel<real>, dim3(cdiv(a.n[0], bx), cdiv(a.n[1], IROWS), a.n[2]), dim3(bx), 0, st, a);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

}  // namespace gm

using namespace gm;

static bool map_ok(const gm_map3& m, const int n[3]) {
  for (int d = 0; d < 3; ++d)
    if (!m.elem[d] || !m.w[d] || m.n[d] != n[d]) return false;
  return m.src_nx > 1 && m.src_ny > 1;
}

extern "C" int gm_interp(const gm_interp_args* g, void* stream) {
  if (!g || !g->out || g->nterms < 1 || g->nterms > 3) return GM_ERR_ARG;
  for (int d = 0; d < 3; ++d)
    if (g->n[d] < 1 || g->n[d] > 65535) return GM_ERR_ARG;  // rows and planes index the launch grid
  for (int q = 0; q < g->nterms; ++q)
    if (!g->src[q] || !map_ok(g->map[q], g->n) || g->src[q] == g->out) return GM_ERR_ARG;
  if (g->out_term && (g->which_term < 0 || g->which_term >= g->nterms)) return GM_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (g->dtype == GM_F32) return do_interp<float>(g, st);
  if (g->dtype == GM_F64) return do_interp<double>(g, st);
  return GM_ERR_ARG;
}

extern "C" int gm_interp_matrix(int dtype, const gm_map3* m, void* Nc, int* node, void* stream) {
  if (!m || !Nc || !node || !map_ok(*m, m->n)) return GM_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  const long long tot = (long long)m->n[0] * m->n[1] * m->n[2];
  if (dtype == GM_F32)
    interp_matrix_kernel<float><<<grid_for(tot), 256, 0, st>>>(make_map3<float>(*m), m->n[0], m->n[1], m->n[2],
                                                                (float*)Nc, node);
  else if (dtype == GM_F64)
    interp_matrix_kernel<double><<<grid_for(tot), 256, 0, st>>>(make_map3<double>(*m), m->n[0], m->n[1], m->n[2],
                                                                 (double*)Nc, node);
  else
    return GM_ERR_ARG;
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_interp_w_matrix(int dtype, const void* Nc, const int* node, const void* T, void* out, long long n,
                                  void* stream) {
  if (!Nc || !node || !T || !out || n < 0) return GM_ERR_ARG;
  if (n == 0) return GM_OK;
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == GM_F32)
    w_matrix_kernel<float><<<grid_for(n), 256, 0, st>>>((const float*)Nc, node, (const float*)T, (float*)out, n);
  else if (dtype == GM_F64)
    w_matrix_kernel<double><<<grid_for(n), 256, 0, st>>>((const double*)Nc, node, (const double*)T, (double*)out, n);
  else
    return GM_ERR_ARG;
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_restrict(const gm_restrict_args* g, void* stream) {
  if (!g || !g->fine || !g->coarse || !map_ok(g->map, g->n) || !g->cidx[0] || !g->cidx[1] || !g->cidx[2])
    return GM_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  const long long tot = (long long)g->n[0] * g->n[1] * g->n[2];
  if (tot == 0) return GM_OK;
  if (tot >= (1LL << 31)) return GM_ERR_TOO_LARGE;
  if (g->dtype == GM_F32)
    launch_k(restrict_kernel<float>, dim3(grid_for(tot)), dim3(256), 0, st, g->n[0], g->n[1], g->n[2],
             make_map3<float>(g->map), g->cidx[0], g->cidx[1], g->cidx[2], g->cnx, g->cny, (const float*)g->fine,
             (float*)g->coarse);
  else if (g->dtype == GM_F64)
    launch_k(restrict_kernel<double>, dim3(grid_for(tot)), dim3(256), 0, st, g->n[0], g->n[1], g->n[2],
             make_map3<double>(g->map), g->cidx[0], g->cidx[1], g->cidx[2], g->cnx, g->cny, (const double*)g->fine,
             (double*)g->coarse);
  else
    return GM_ERR_ARG;
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

template <typename real>
static int do_tprime(const gm_tprime_args* g, cudaStream_t st) {
  TprimeK<real> a;
  for (int d = 0; d < 3; ++d) {
    a.n[d] = g->n[d];
    a.cf0[d] = g->cf0[d];
    a.cf1[d] = g->cf1[d];
    a.c_of_f[d] = g->c_of_f[d];
  }
  a.cmap = make_map3<real>(g->cmap);
  a.cnx = g->cnx;
  a.cny = g->cny;
  a.fine = (const real*)g->fine;
  a.coarse = (real*)g->coarse;
  a.out = (real*)g->out;
  const int bx = a.n[0] <= 256 ? 32 * cdiv(a.n[0], 32) : 256;
  launch_k(tprime_inject_kernel<real>, dim3(cdiv(a.n[0], bx), cdiv(a.n[1], TROWS), a.n[2]), dim3(bx), 0, st, a);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_tprime_inject(const gm_tprime_args* g, void* stream) {
  if (!g || !g->fine || !g->coarse || !g->out || g->out == g->fine || !map_ok(g->cmap, g->n) ||
      g->cnx != g->cmap.src_nx || g->cny != g->cmap.src_ny)
    return GM_ERR_ARG;
  for (int d = 0; d < 3; ++d)
    if (g->n[d] < 1 || g->n[d] > 65535 || !g->cf0[d] || !g->cf1[d] || !g->c_of_f[d]) return GM_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (g->dtype == GM_F32) return do_tprime<float>(g, st);
  if (g->dtype == GM_F64) return do_tprime<double>(g, st);
  return GM_ERR_ARG;
}

extern "C" int gm_restrict_s1(const gm_restrict_s1_args* g, void* stream) {
  if (!g || !g->fine_ph || !g->coarse_ph || !map_ok(g->map, g->n) || !g->cidx[0] || !g->cidx[1] || !g->cidx[2])
    return GM_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  const long long tot = (long long)g->n[0] * g->n[1] * g->n[2];
  if (tot == 0 && g->substrate <= 0) return GM_OK;
  const long long work = tot > g->substrate ? tot : g->substrate;
  if (g->dtype == GM_F32)
    launch_k(restrict_s1_kernel<float>, dim3(grid_for(work)), dim3(256), 0, st,
        g->n[0], g->n[1], g->n[2], make_map3<float>(g->map), g->cidx[0], g->cidx[1], g->cidx[2], g->cnx, g->cny,
        g->fine_ph, g->map.src_nx, g->map.src_ny, g->coarse_ph, g->substrate);
  else if (g->dtype == GM_F64)
    launch_k(restrict_s1_kernel<double>, dim3(grid_for(work)), dim3(256), 0, st,
        g->n[0], g->n[1], g->n[2], make_map3<double>(g->map), g->cidx[0], g->cidx[1], g->cidx[2], g->cnx, g->cny,
        g->fine_ph, g->map.src_nx, g->map.src_ny, g->coarse_ph, g->substrate);
  else
    return GM_ERR_ARG;
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_l0_gather(const gm_l0_args* g, void* stream) {
  if (!g || !g->l0_bits || !g->ph || !g->idx[0] || !g->idx[1] || !g->idx[2] || g->ph == g->prev_ph ||
      g->l0_nx < 1 || g->l0_ny < 1)
    return GM_ERR_ARG;
  const long long tot = (long long)g->n[0] * g->n[1] * g->n[2];
  if (tot == 0) return GM_OK;
  l0_gather_kernel<<<grid_for(tot), 256, 0, (cudaStream_t)stream>>>(
      g->n[0], g->n[1], g->n[2], g->idx[0], g->idx[1], g->idx[2], g->l0_nx, g->l0_ny, g->l0_bits, g->ph, g->prev_ph,
      g->prev_lo[0], g->prev_lo[1], g->prev_lo[2], g->prev_n[0], g->prev_n[1], g->prev_n[2]);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_l0_scatter(const gm_l0_args* g, void* stream) {
  if (!g || !g->l0_bits || !g->ph || !g->idx[0] || !g->idx[1] || !g->idx[2] || g->l0_nx < 1 || g->l0_ny < 1)
    return GM_ERR_ARG;
  const long long tot = (long long)g->n[0] * g->n[1] * g->n[2];
  if (tot == 0) return GM_OK;
  l0_scatter_kernel<<<grid_for(tot), 256, 0, (cudaStream_t)stream>>>(g->n[0], g->n[1], g->n[2], g->idx[0], g->idx[1],
                                                                      g->idx[2], g->l0_nx, g->l0_ny, g->l0_bits, g->ph);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" long long gm_l0_words(long long nx, long long ny, long long nz) {
  if (nx < 1 || ny < 1 || nz < 1) return -1;
  return l0_words_per_row(nx) * ny * nz;
}

extern "C" int gm_l0_fill(uint32_t* l0_bits, long long nx, long long ny, long long nz, long long first,
                          long long last, int value, void* stream) {
  if (!l0_bits || nx < 1 || ny < 1 || nz < 1 || first < 0 || last > nx * ny * nz || first > last) return GM_ERR_ARG;
  if (first == last) return GM_OK;
  l0_fill_kernel<<<grid_for(l0_words_per_row(nx) * ny * nz), 256, 0, (cudaStream_t)stream>>>(nx, ny, nz, first, last,
                                                                                              l0_bits, value);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

// T = max(T, lo) (the reference's jnp.maximum(T_amb, T) after computeSolutions,
// stepGOMELT :2360-2362, :2380-2382).
template <typename real>
__global__ void clamp_kernel(real* T, long long n, real lo) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    T[i] = fmax(T[i], lo);
}

extern "C" int gm_clamp_min(int dtype, void* T, long long n, double lo, void* stream) {
  if (!T || n < 0) return GM_ERR_ARG;
  if (n == 0) return GM_OK;
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == GM_F32)
    clamp_kernel<float><<<grid_for(n), 256, 0, st>>>((float*)T, n, (float)lo);
  else if (dtype == GM_F64)
    clamp_kernel<double><<<grid_for(n), 256, 0, st>>>((double*)T, n, lo);
  else
    return GM_ERR_ARG;
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

// Prolongation onto the Dirichlet ring of a fine level (faces x0, x1, y0, y1
// and the bottom plane; computeL2Temperature :2937-2955, computeSolutions_L3
// :3039-3052): outA = I(srcA), outB = I(srcB) at the ring nodes only, written
// at their node ids in full-size arrays.  The reference blends the coarse
// field first, I(alpha*Tn + beta*To); the level kernel forms
// alpha*I(Tn) + beta*I(To), the same linear combination, so both
// prolongations are computed once for all fine steps that share Tn and To.
template <typename real>
__global__ void ring_kernel(int nx, int ny, int nz, const Map3<real> m, const real* srcA, const real* srcB,
                            real* outA, real* outB) {
  pdl_begin();
  // ring nodes in the order bottom plane, x faces, y faces, with x or y the
  // fastest index inside each plane (contiguous stores on the bottom plane
  // and the y faces); counts < 2^31 (checked by the caller)
  const int nb = nx * ny;                               // bottom plane
  const int nxf = 2 * ny * (nz - 1);                    // x faces above the bottom
  const int nyi = nx > 2 ? nx - 2 : 0;
  const int nyf = 2 * nyi * (nz - 1);                   // y faces, x interior
  const int tot = nb + nxf + nyf;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < tot; r += gridDim.x * blockDim.x) {
    int ix, iy, iz;
    if (r < nb) {
      ix = r % nx;
      iy = r / nx;
      iz = 0;
    } else if (r < nb + nxf) {
      const int q = r - nb, q2 = q / ny;
      iy = q - q2 * ny;
      ix = (q2 & 1) ? nx - 1 : 0;
      iz = 1 + (q2 >> 1);
    } else {
      const int q = r - nb - nxf, q2 = q / nyi;
      ix = 1 + (q - q2 * nyi);
      iy = (q2 & 1) ? ny - 1 : 0;
      iz = 1 + (q2 >> 1);
    }
    real w8[8];
    const int b = map3_weights(m, ix, iy, iz, w8);
    const int sx = 1, sy = m.src_nx, sz = m.src_nx * m.src_ny;
    const int off[8] = {0, sx, sx + sy, sy, sz, sx + sz, sx + sy + sz, sy + sz};
    real a = 0, c = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      a += w8[j] * srcA[b + off[j]];
      if (srcB) c += w8[j] * srcB[b + off[j]];
    }
    const int id = ix + iy * nx + iz * nb;
    outA[id] = a;
    if (outB) outB[id] = c;
  }
}

extern "C" int gm_ring_prolong(const gm_ring_args* g, void* stream) {
  if (!g || !g->srcA || !g->outA || (g->srcB == nullptr) != (g->outB == nullptr)) return GM_ERR_ARG;
  if (g->nodes[0] < 2 || g->nodes[1] < 2 || g->nodes[2] < 2 || !map_ok(g->map, g->nodes)) return GM_ERR_ARG;
  if ((long long)g->nodes[0] * g->nodes[1] * g->nodes[2] >= (1LL << 31)) return GM_ERR_TOO_LARGE;
  const long long nx = g->nodes[0], ny = g->nodes[1], nz = g->nodes[2];
  const long long tot = nx * ny + 2 * ny * (nz - 1) + 2 * (nx - 2) * (nz - 1);
  cudaStream_t st = (cudaStream_t)stream;
  if (g->dtype == GM_F32)
    launch_k(ring_kernel<float>, dim3(grid_for(tot)), dim3(256), 0, st, g->nodes[0], g->nodes[1], g->nodes[2],
             make_map3<float>(g->map), (const float*)g->srcA, (const float*)g->srcB, (float*)g->outA,
             (float*)g->outB);
  else if (g->dtype == GM_F64)
    launch_k(ring_kernel<double>, dim3(grid_for(tot)), dim3(256), 0, st, g->nodes[0], g->nodes[1], g->nodes[2],
             make_map3<double>(g->map), (const double*)g->srcA, (const double*)g->srcB, (double*)g->outA,
             (double*)g->outB);
  else
    return GM_ERR_ARG;
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}
