// BF16 tensor-core kernels of the Level-3 surrogate (a 3-D convolutional
// U-Net that predicts the Level-3 field after one Level-2 step).  No
// counterpart in the reference.
//
// Activations are channels-last BF16 tensors [B][Z][Y][X][C] (C innermost),
// optionally a channel slice (offset, stride) of a wider tensor so that skip
// connections concatenate without copies of the consumer's input.  Weights of
// a 3x3x3 convolution are BF16 [27][Cout][Cin] (tap = dx + 3 dy + 9 dz,
// d in {0,1,2} for offsets -1, 0, +1), with an FP32 master copy for Adam.
//
// conv3_kernel: implicit GEMM, M = voxels, N = Cout, K = 27 * Cin, on
// mma.sync m16n8k16 (BF16 in, FP32 accumulate).  A warp owns 16 voxels and
// all Cout columns; the CTA stages the weights of one tap in shared memory.
// The same kernel computes the data gradient dX[u] = sum_tap dY[u - d(tap)]
// W[tap]^T (tap offsets negated, weights laid out [27][Cin][Cout]).
// wgrad_kernel: dW[tap][co][ci] = sum_v dY[v][co] X[v + off(tap)][ci], the
// voxel sum split over CTAs into FP32 partials reduced in a fixed order.
#include <cuda_bf16.h>
#include <stdint.h>

#include "gm_common.cuh"

namespace gm {

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ uint32_t pack_raw(uint16_t lo, uint16_t hi) { return (uint32_t)lo | ((uint32_t)hi << 16); }
__device__ __forceinline__ float bf2f(uint16_t u) { return __uint_as_float((uint32_t)u << 16); }

struct Grid5 {
  int B, X, Y, Z;
};

__device__ __forceinline__ void vox_xyz(const Grid5& g, long long v, int& x, int& y, int& z, long long& base) {
  x = (int)(v % g.X);
  long long r = v / g.X;
  y = (int)(r % g.Y);
  r /= g.Y;
  z = (int)(r % g.Z);
  base = v - x - (long long)g.X * (y + (long long)g.Y * z);  // first voxel of this sample
}

// ---------------------------------------------------------------------------
// 3x3x3 convolution (forward or data gradient).
// ---------------------------------------------------------------------------
struct ConvK {
  Grid5 g;
  int cin, in_stride, in_off;     // input channels (multiple of 16), slice of a tensor of in_stride channels
  int out_stride, out_off;        // output slice
  int mask_stride, mask_off;      // optional mask slice (output *= mask > 0)
  int mirror;                     // 1: data gradient (tap offsets negated)
  int relu;
  const uint16_t* in;
  const uint16_t* w;              // [27][COUT][cin]
  const float* bias;              // [COUT] or null
  const uint16_t* mask;           // or null
  uint16_t* out;
};

constexpr int CV_WARPS = 8;

// Voxel rows per warp: MT m16 tiles, so that a warp's accumulators stay at
// 64 registers (MT * COUT / 8 * 4) and every weight fragment read from shared
// memory feeds MT MMAs.
template <int COUT>
struct ConvShape {
  static constexpr int NT = COUT / 8;
  static constexpr int MT = NT >= 16 ? 1 : (16 / NT > 4 ? 4 : 16 / NT);
  static constexpr int ROWS = 16 * MT;  // voxels per warp
};

template <int COUT>
__global__ void __launch_bounds__(CV_WARPS * 32) conv3_kernel(const ConvK a) {
  constexpr int NT = ConvShape<COUT>::NT, MT = ConvShape<COUT>::MT;
  extern __shared__ uint32_t smw[];  // one tap: COUT rows of (cin + 8) bf16
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int rs = (a.cin + 8) / 2;  // row stride in 32-bit words
  const long long V = (long long)a.g.B * a.g.X * a.g.Y * a.g.Z;
  const long long v0 = ((long long)blockIdx.x * CV_WARPS + warp) * (16 * MT);
  // per row: packed (x, y, z) (10 bits each; -1 when the row is past the end)
  // and the first voxel of its sample (voxel counts < 2^31)
  int xyz[MT][2], br[MT][2];
#pragma unroll
  for (int m = 0; m < MT; ++m)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const long long v = v0 + 16 * m + g + 8 * h;
      int x, y, z;
      long long b;
      vox_xyz(a.g, v < V ? v : 0, x, y, z, b);
      xyz[m][h] = v < V ? (x | (y << 10) | (z << 20)) : -1;
      br[m][h] = (int)b;
    }
  float acc[MT][NT][4];
#pragma unroll
  for (int m = 0; m < MT; ++m)
#pragma unroll
    for (int n = 0; n < NT; ++n) acc[m][n][0] = acc[m][n][1] = acc[m][n][2] = acc[m][n][3] = 0.f;
  const int kc = a.cin / 16;
  for (int tap = 0; tap < 27; ++tap) {
    __syncthreads();  // previous tap's weights are no longer read
    // data gradient: dX[u] = sum_tap dY[u - d(tap)] W[tap]^T, same weight tap, offset negated
    const uint32_t* wsrc = reinterpret_cast<const uint32_t*>(a.w + (long long)tap * COUT * a.cin);
    for (int i = threadIdx.x; i < COUT * (a.cin / 2); i += blockDim.x) {
      const int r = i / (a.cin / 2), c = i - r * (a.cin / 2);
      smw[r * rs + c] = wsrc[i];
    }
    __syncthreads();
    const int dx = tap % 3 - 1, dy = (tap / 3) % 3 - 1, dz = tap / 9 - 1;
    const int sx = a.mirror ? -dx : dx, sy = a.mirror ? -dy : dy, sz = a.mirror ? -dz : dz;
    const uint32_t* src[MT][2];
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int p = xyz[m][h];
        const int x = (p & 1023) + sx, y = ((p >> 10) & 1023) + sy, z = ((p >> 20) & 1023) + sz;
        const bool in = p >= 0 && x >= 0 && x < a.g.X && y >= 0 && y < a.g.Y && z >= 0 && z < a.g.Z;
        const long long nb = br[m][h] + x + (long long)a.g.X * (y + (long long)a.g.Y * z);
        src[m][h] = in ? reinterpret_cast<const uint32_t*>(a.in + nb * a.in_stride + a.in_off) : nullptr;
      }
    for (int c = 0; c < kc; ++c) {
      uint32_t af[MT][4];
#pragma unroll
      for (int m = 0; m < MT; ++m) {
        af[m][0] = src[m][0] ? src[m][0][c * 8 + t] : 0u;
        af[m][1] = src[m][1] ? src[m][1][c * 8 + t] : 0u;
        af[m][2] = src[m][0] ? src[m][0][c * 8 + 4 + t] : 0u;
        af[m][3] = src[m][1] ? src[m][1][c * 8 + 4 + t] : 0u;
      }
#pragma unroll
      for (int n = 0; n < NT; ++n) {
        const uint32_t* wr = smw + (n * 8 + g) * rs + c * 8;
        const uint32_t b0 = wr[t], b1 = wr[4 + t];
#pragma unroll
        for (int m = 0; m < MT; ++m) mma16816(acc[m][n], af[m], b0, b1);
      }
    }
  }
  // epilogue: bias, ReLU, mask, BF16 store
#pragma unroll
  for (int m = 0; m < MT; ++m)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (xyz[m][h] < 0) continue;
      const long long v = v0 + 16 * m + g + 8 * h;
#pragma unroll
      for (int n = 0; n < NT; ++n) {
        const int co = n * 8 + 2 * t;
        float y0 = acc[m][n][2 * h], y1 = acc[m][n][2 * h + 1];
        if (a.bias) {
          y0 += a.bias[co];
          y1 += a.bias[co + 1];
        }
        if (a.relu) {
          y0 = fmaxf(y0, 0.f);
          y1 = fmaxf(y1, 0.f);
        }
        if (a.mask) {
          const uint32_t mk = *reinterpret_cast<const uint32_t*>(a.mask + v * a.mask_stride + a.mask_off + co);
          if (bf2f((uint16_t)(mk & 0xffffu)) <= 0.f) y0 = 0.f;
          if (bf2f((uint16_t)(mk >> 16)) <= 0.f) y1 = 0.f;
        }
        *reinterpret_cast<uint32_t*>(a.out + v * a.out_stride + a.out_off + co) = pack_bf16(y0, y1);
      }
    }
}

// ---------------------------------------------------------------------------
// Weight gradient.  CTA = (tap, voxel chunk); warps tile (co: 16 rows) x
// (ci: CI_T columns).  Staged per 32 voxels: dY tile [32][COUT] and the
// shifted X tile [32][cin] in shared memory; fragments are read with 16-bit
// loads (K = voxel is the strided dimension of both operands).
// ---------------------------------------------------------------------------
struct WgradK {
  Grid5 g;
  int cin, cout;
  int in_stride, in_off, dy_stride, dy_off;
  const uint16_t* in;
  const uint16_t* dy;
  float* part;  // [nsplit][27][cout][cin]
  long long chunk;
  int nsplit;
};

constexpr int WG_WARPS = 8;
constexpr int WG_KV = 64;  // voxels staged per step

// Four 8x8 BF16 blocks from shared memory, transposed (thread (g, t) receives
// rows 2t, 2t+1 of column g of each block): the K-strided operands of the
// weight-gradient GEMM as mma fragments.
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const uint16_t* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a));
}

// Warp tiles: 16 output channels (co) x NB8 * 8 input channels (ci); up to
// four tiles per warp, statically indexed.  Voxel tiles of dY and the
// tap-shifted X are staged with rows padded to a 16-byte multiple, so every
// fragment comes from one ldmatrix.trans.
template <int NB8>
__global__ void __launch_bounds__(WG_WARPS * 32) wgrad_kernel(const WgradK a) {
  extern __shared__ __align__(16) uint16_t sm[];
  const int tap = blockIdx.y, split = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int cin = a.cin, cout = a.cout;
  const int sdy = cout + 8, sx = cin + 8;  // row strides (bf16), multiples of 8
  uint16_t* sDy = sm;
  uint16_t* sX = sm + WG_KV * sdy;
  const long long V = (long long)a.g.B * a.g.X * a.g.Y * a.g.Z;
  const long long vb = (long long)split * a.chunk, ve = min(V, vb + a.chunk);
  const int dx = tap % 3 - 1, dy = (tap / 3) % 3 - 1, dz = tap / 9 - 1;
  const int mt = cout / 16, ntile = cin / (NB8 * 8), tiles = mt * ntile;
  float acc[4][NB8][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int n = 0; n < NB8; ++n) acc[i][n][0] = acc[i][n][1] = acc[i][n][2] = acc[i][n][3] = 0.f;
  // ldmatrix row addresses: lane l supplies row (l & 7) of block (l >> 3)
  const int lr = lane & 7, lb = lane >> 3;
  for (long long v0 = vb; v0 < ve; v0 += WG_KV) {
    __syncthreads();
    for (int r = warp; r < WG_KV; r += WG_WARPS) {
      const long long v = v0 + r;
      const bool vin = v < ve;
      const uint32_t* srcd = vin ? reinterpret_cast<const uint32_t*>(a.dy + v * a.dy_stride + a.dy_off) : nullptr;
      const uint32_t* srcx = nullptr;
      if (vin) {
        int x, y, z;
        long long base;
        vox_xyz(a.g, v, x, y, z, base);
        x += dx;
        y += dy;
        z += dz;
        if (x >= 0 && x < a.g.X && y >= 0 && y < a.g.Y && z >= 0 && z < a.g.Z)
          srcx = reinterpret_cast<const uint32_t*>(
              a.in + (base + x + (long long)a.g.X * (y + (long long)a.g.Y * z)) * a.in_stride + a.in_off);
      }
      uint32_t* dd = reinterpret_cast<uint32_t*>(sDy + r * sdy);
      uint32_t* dxs = reinterpret_cast<uint32_t*>(sX + r * sx);
      for (int c = lane; c < cout / 2; c += 32) dd[c] = srcd ? srcd[c] : 0u;
      for (int c = lane; c < cin / 2; c += 32) dxs[c] = srcx ? srcx[c] : 0u;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < WG_KV; kk += 16) {
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        const int tile = warp + s * WG_WARPS;
        if (tile >= tiles) continue;
        const int m0 = (tile % mt) * 16, n0 = (tile / mt) * (NB8 * 8);
        // A[co][v] = dY[v][co]: blocks (co 0-7 | 8-15) x (v 0-7 | 8-15) -> a0..a3
        uint32_t af[4];
        ldsm_x4_t(af, sDy + (kk + lr + 8 * (lb >> 1)) * sdy + m0 + 8 * (lb & 1));
#pragma unroll
        for (int n = 0; n < NB8; n += 2) {
          // B[v][ci] = X[v][ci]: blocks (v 0-7 | 8-15) x (ci n | n+1) -> b0, b1 of n and n+1
          uint32_t bf[4];
          ldsm_x4_t(bf, sX + (kk + lr + 8 * (lb & 1)) * sx + n0 + 8 * (n + (lb >> 1)));
          mma16816(acc[s][n], af, bf[0], bf[1]);
          mma16816(acc[s][n + 1], af, bf[2], bf[3]);
        }
      }
    }
  }
  float* P = a.part + ((long long)split * 27 + tap) * cout * cin;
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const int tile = warp + s * WG_WARPS;
    if (tile >= tiles) continue;
    const int m0 = (tile % mt) * 16, n0 = (tile / mt) * (NB8 * 8);
#pragma unroll
    for (int n = 0; n < NB8; ++n) {
      const int ci = n0 + n * 8 + 2 * t;
      P[(m0 + g) * cin + ci] = acc[s][n][0];
      P[(m0 + g) * cin + ci + 1] = acc[s][n][1];
      P[(m0 + g + 8) * cin + ci] = acc[s][n][2];
      P[(m0 + g + 8) * cin + ci + 1] = acc[s][n][3];
    }
  }
}

__global__ void sum_splits_kernel(const float* part, int nsplit, long long n, float* out, float scale) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int k = 0; k < nsplit; ++k) s += part[k * n + i];
    out[i] = s * scale;
  }
}

// dbias[c] = sum_v dY[v][c]: per-block partials over voxel chunks, then a
// fixed-order sum.
__global__ void bias_grad_kernel(long long V, int C, const uint16_t* dy, int stride, int off, long long chunk,
                                 float* part) {
  const long long vb = blockIdx.x * chunk, ve = min(V, vb + chunk);
  for (int c = threadIdx.x; c < C; c += blockDim.x) {
    float s = 0.f;
    for (long long v = vb; v < ve; ++v) s += bf2f(dy[v * stride + off + c]);
    part[(long long)blockIdx.x * C + c] = s;
  }
}

// ---------------------------------------------------------------------------
// 2x average pooling / nearest upsampling on channel slices, and backward.
// ---------------------------------------------------------------------------
__global__ void pool2_kernel(Grid5 g, int C, const uint16_t* in, int is, int io, uint16_t* out, int os, int oo,
                             int backward) {
  // forward: out grid = g/2; backward: in = dOut (coarse), out = dIn (fine, g)
  const int Xc = g.X / 2, Yc = g.Y / 2, Zc = g.Z / 2;
  if (!backward) {
    const long long n = (long long)g.B * Xc * Yc * Zc * C;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
      const int c = (int)(i % C);
      long long v = i / C;
      const int x = (int)(v % Xc), y = (int)((v / Xc) % Yc), z = (int)((v / ((long long)Xc * Yc)) % Zc);
      const long long b = v / ((long long)Xc * Yc * Zc);
      float s = 0.f;
      for (int k = 0; k < 8; ++k) {
        const long long f = (((b * g.Z + 2 * z + (k >> 2)) * g.Y + 2 * y + ((k >> 1) & 1)) * g.X) + 2 * x + (k & 1);
        s += bf2f(in[f * is + io + c]);
      }
      __nv_bfloat16 r = __float2bfloat16_rn(0.125f * s);
      out[v * os + oo + c] = *reinterpret_cast<uint16_t*>(&r);
    }
  } else {
    const long long n = (long long)g.B * g.X * g.Y * g.Z * C;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
      const int c = (int)(i % C);
      long long f = i / C;
      const int x = (int)(f % g.X), y = (int)((f / g.X) % g.Y), z = (int)((f / ((long long)g.X * g.Y)) % g.Z);
      const long long b = f / ((long long)g.X * g.Y * g.Z);
      const long long v = ((b * Zc + z / 2) * Yc + y / 2) * Xc + x / 2;
      __nv_bfloat16 r = __float2bfloat16_rn(0.125f * bf2f(in[v * is + io + c]));
      out[f * os + oo + c] = *reinterpret_cast<uint16_t*>(&r);
    }
  }
}

// forward: fine[f] = coarse[f/2]; backward: dCoarse[v] = sum of the 8 dFine.
__global__ void up2_kernel(Grid5 g, int C, const uint16_t* in, int is, int io, uint16_t* out, int os, int oo,
                           int backward) {
  const int Xc = g.X / 2, Yc = g.Y / 2, Zc = g.Z / 2;
  if (!backward) {
    const long long n = (long long)g.B * g.X * g.Y * g.Z * C;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
      const int c = (int)(i % C);
      long long f = i / C;
      const int x = (int)(f % g.X), y = (int)((f / g.X) % g.Y), z = (int)((f / ((long long)g.X * g.Y)) % g.Z);
      const long long b = f / ((long long)g.X * g.Y * g.Z);
      const long long v = ((b * Zc + z / 2) * Yc + y / 2) * Xc + x / 2;
      out[f * os + oo + c] = in[v * is + io + c];
    }
  } else {
    const long long n = (long long)g.B * Xc * Yc * Zc * C;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
      const int c = (int)(i % C);
      long long v = i / C;
      const int x = (int)(v % Xc), y = (int)((v / Xc) % Yc), z = (int)((v / ((long long)Xc * Yc)) % Zc);
      const long long b = v / ((long long)Xc * Yc * Zc);
      float s = 0.f;
      for (int k = 0; k < 8; ++k) {
        const long long f = (((b * g.Z + 2 * z + (k >> 2)) * g.Y + 2 * y + ((k >> 1) & 1)) * g.X) + 2 * x + (k & 1);
        s += bf2f(in[f * is + io + c]);
      }
      __nv_bfloat16 r = __float2bfloat16_rn(s);
      out[v * os + oo + c] = *reinterpret_cast<uint16_t*>(&r);
    }
  }
}

// The same two kernels eight channels (16 bytes) a thread, for channel counts,
// slice offsets and strides that are multiples of 8 and 16-byte aligned
// bases (every tensor of the surrogate's U-Net); per channel the arithmetic
// and its order are those of the element-wise forms (same bits).  Voxel ids
// are 32-bit (grids below 2^31 voxels).
__device__ __forceinline__ void bf8_to_f(const uint4 q, float (&f)[8]) {
  const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    f[2 * i] = __uint_as_float(w[i] << 16);
    f[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
  }
}
__device__ __forceinline__ uint4 f_to_bf8(const float (&f)[8]) {
  uint32_t w[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    __nv_bfloat162 v = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
    w[i] = *reinterpret_cast<uint32_t*>(&v);
  }
  return make_uint4(w[0], w[1], w[2], w[3]);
}

// pool (mode 0) / up (mode 1), forward or backward, 8 channels a thread.
// Fine-to-coarse sums (pool forward, up backward) add the 8 fine voxels in
// the order k = 0..7 and scale by `scale` (0.125 or 1); coarse-to-fine copies
// (up forward) or scaled copies (pool backward, scale 0.125) otherwise.
__global__ void resample8_kernel(Grid5 g, int C8, const uint16_t* in, int is, int io, uint16_t* out, int os, int oo,
                                 int gather, float scale, int copy) {
  const unsigned Xc = g.X / 2, Yc = g.Y / 2, Zc = g.Z / 2;
  if (gather) {  // out on the coarse grid, sum of 8 fine voxels
    const unsigned n = (unsigned)g.B * Xc * Yc * Zc * C8;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      const unsigned c8 = i % C8, v = i / C8;
      const unsigned x = v % Xc, y = (v / Xc) % Yc, t = v / (Xc * Yc), z = t % Zc, b = t / Zc;
      float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const unsigned f = ((b * g.Z + 2 * z + (k >> 2)) * g.Y + 2 * y + ((k >> 1) & 1)) * g.X + 2 * x + (k & 1);
        float e[8];
        bf8_to_f(__ldg(reinterpret_cast<const uint4*>(in + (size_t)f * is + io) + c8), e);
#pragma unroll
        for (int q = 0; q < 8; ++q) s[q] += e[q];
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) s[q] = scale * s[q];
      reinterpret_cast<uint4*>(out + (size_t)v * os + oo)[c8] = f_to_bf8(s);
    }
  } else {  // out on the fine grid from its coarse voxel
    const unsigned n = (unsigned)g.B * g.X * g.Y * g.Z * C8;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      const unsigned c8 = i % C8, f = i / C8;
      const unsigned x = f % g.X, y = (f / g.X) % g.Y, t = f / (g.X * g.Y), z = t % g.Z, b = t / g.Z;
      const unsigned v = ((b * Zc + z / 2) * Yc + y / 2) * Xc + x / 2;
      uint4 q = __ldg(reinterpret_cast<const uint4*>(in + (size_t)v * is + io) + c8);
      if (!copy) {
        float e[8];
        bf8_to_f(q, e);
#pragma unroll
        for (int k = 0; k < 8; ++k) e[k] = scale * e[k];
        q = f_to_bf8(e);
      }
      reinterpret_cast<uint4*>(out + (size_t)f * os + oo)[c8] = q;
    }
  }
}

static bool vec8_ok(const int grid[4], int C, const void* in, int is, int io, const void* out, int os, int oo) {
  const long long V = (long long)grid[0] * grid[1] * grid[2] * grid[3];
  return C % 8 == 0 && is % 8 == 0 && io % 8 == 0 && os % 8 == 0 && oo % 8 == 0 &&
         !(((uintptr_t)in | (uintptr_t)out) & 15) && V * (C / 8) < (1LL << 31) && V * (long long)(is > os ? is : os) < (1LL << 62);
}

// b += a (where mask > 0, if a mask is given): the gradient of a tensor used
// twice, the second path's gradient passed through the ReLU of its producer.
__global__ void add_slice_kernel(long long V, int C, const uint16_t* a, int as, int ao, uint16_t* b, int bs, int bo,
                                 const uint16_t* m, int ms, int mo) {
  const long long n = V * C;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long v = i / C;
    const int c = (int)(i % C);
    const float av = (m && bf2f(m[v * ms + mo + c]) <= 0.f) ? 0.f : bf2f(a[v * as + ao + c]);
    __nv_bfloat16 r = __float2bfloat16_rn(av + bf2f(b[v * bs + bo + c]));
    b[v * bs + bo + c] = *reinterpret_cast<uint16_t*>(&r);
  }
}

// ---------------------------------------------------------------------------
// Head: 1x1x1 convolution C -> 1 (FP32 output), its gradients, MSE loss.
// ---------------------------------------------------------------------------
__global__ void head_fwd_kernel(long long V, int C, const uint16_t* in, int is, int io, const float* w, float b,
                                float* out) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    float s = b;
    for (int c = 0; c < C; ++c) s += w[c] * bf2f(in[v * is + io + c]);
    out[v] = s;
  }
}

// dOut = 2 (pred - target) m / count (mask m: voxels in the loss); dIn[v][c] =
// dOut[v] w[c] where the head's (ReLU) input is positive; per-block partials
// of dW[c], db and the loss, reduced in a fixed order.
constexpr int HB_THREADS = 128;
constexpr int HB_CMAX = 32;
__global__ void __launch_bounds__(HB_THREADS) head_bwd_kernel(long long V, int C, const uint16_t* in, int is, int io,
                                                              const float* w, const float* pred, const float* target,
                                                              const float* lmask, float inv_count, uint16_t* din,
                                                              int ds, int dof, long long chunk, float* part) {
  __shared__ float sp[HB_THREADS][HB_CMAX + 3];
  float acc[HB_CMAX + 2];
#pragma unroll
  for (int c = 0; c < HB_CMAX + 2; ++c) acc[c] = 0.f;
  const long long vb = blockIdx.x * chunk, ve = min(V, vb + chunk);
  for (long long v = vb + threadIdx.x; v < ve; v += blockDim.x) {
    const float m = lmask ? lmask[v] : 1.f;
    const float e = (pred[v] - target[v]) * m;
    const float go = 2.f * e * inv_count;
#pragma unroll
    for (int c = 0; c < HB_CMAX; ++c) {
      if (c >= C) break;
      const float x = bf2f(in[v * is + io + c]);
      acc[c] += go * x;
      __nv_bfloat16 r = __float2bfloat16_rn(x > 0.f ? go * w[c] : 0.f);
      din[v * ds + dof + c] = *reinterpret_cast<uint16_t*>(&r);
    }
    acc[HB_CMAX] += go;
    acc[HB_CMAX + 1] += e * e * inv_count;
  }
#pragma unroll
  for (int c = 0; c < HB_CMAX + 2; ++c) sp[threadIdx.x][c] = acc[c];
  __syncthreads();
  for (int c = threadIdx.x; c < C + 2; c += blockDim.x) {
    const int src = c < C ? c : HB_CMAX + (c - C);
    float s = 0.f;
    for (int k = 0; k < HB_THREADS; ++k) s += sp[k][src];
    part[(long long)blockIdx.x * (C + 2) + c] = s;
  }
}

// ---------------------------------------------------------------------------
// Adam on an FP32 master copy; writes the BF16 copy (optionally transposed to
// [27][cin][cout] for the data-gradient convolution).
// ---------------------------------------------------------------------------
__global__ void adam_kernel(long long n, float* w, const float* gr, float* m, float* v, float lr, float b1, float b2,
                            float eps, float c1, float c2, float wd, uint16_t* wb, uint16_t* wt, int cout, int cin) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float gi = gr[i] + wd * w[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) {
      __nv_bfloat16 r = __float2bfloat16_rn(wi);
      const uint16_t u = *reinterpret_cast<uint16_t*>(&r);
      wb[i] = u;
      if (wt) {  // i = (tap * cout + co) * cin + ci  ->  (tap * cin + ci) * cout + co
        const long long tap = i / ((long long)cout * cin);
        const int rem = (int)(i - tap * cout * cin), co = rem / cin, ci = rem - co * cin;
        wt[(tap * cin + ci) * cout + co] = u;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Surrogate input / output on a level window: the network grid is the node
// block ix < X, iy < Y, 1 <= iz <= Z of each sample's window (the bottom
// plane iz = 0 is Dirichlet).  Channels (16, BF16): 0 (I(T2) - T_amb) / S,
// 1 (T3_start - T_amb) / S, 2-3 node offset from the mid-step laser position
// / r_s, 4 P / P_s, 5 v / v_s, 6-15 zero.  Target / prediction: the fine
// correction (T3_end - I(T2)) / S; loss mask: nodes off the Dirichlet ring.
// ---------------------------------------------------------------------------
__global__ void surr_pack_kernel(Grid5 g, int nx, int ny, long long nn, const float* T2i, const float* T3o,
                                 const float* T3n, const double* par, float Tamb, float S, uint16_t* x, float* target,
                                 float* lmask) {
  const long long V = (long long)g.B * g.X * g.Y * g.Z;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    int ix, iy, iz;
    long long base;
    vox_xyz(g, v, ix, iy, iz, base);
    const long long b = v / ((long long)g.X * g.Y * g.Z);
    const long long node = b * nn + ix + (long long)nx * (iy + (long long)ny * (iz + 1));
    const double* q = par + b * 8;  // ox, oy, h, lx, ly, 1/r_s, P/P_s, v/v_s
    const float t2 = T2i[node];
    float ch[6];
    ch[0] = (t2 - Tamb) / S;
    ch[1] = (T3o[node] - Tamb) / S;
    ch[2] = (float)((q[0] + q[2] * ix - q[3]) * q[5]);
    ch[3] = (float)((q[1] + q[2] * iy - q[4]) * q[5]);
    ch[4] = (float)q[6];
    ch[5] = (float)q[7];
    uint32_t* xo = reinterpret_cast<uint32_t*>(x + v * 16);
    xo[0] = pack_bf16(ch[0], ch[1]);
    xo[1] = pack_bf16(ch[2], ch[3]);
    xo[2] = pack_bf16(ch[4], ch[5]);
#pragma unroll
    for (int k = 3; k < 8; ++k) xo[k] = 0u;
    if (target) target[v] = T3n ? (T3n[node] - t2) / S : 0.f;
    if (lmask) lmask[v] = (ix >= 1 && iy >= 1) ? 1.f : 0.f;
  }
}

// T3[node] = I(T2)[node] + S pred[v] on the network grid's nodes off the
// Dirichlet ring; other nodes keep T3.
__global__ void surr_unpack_kernel(Grid5 g, int nx, int ny, long long nn, const float* T2i, const float* pred, float S,
                                   float* T3) {
  const long long V = (long long)g.B * g.X * g.Y * g.Z;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    int ix, iy, iz;
    long long base;
    vox_xyz(g, v, ix, iy, iz, base);
    if (ix < 1 || iy < 1) continue;
    const long long b = v / ((long long)g.X * g.Y * g.Z);
    const long long node = b * nn + ix + (long long)nx * (iy + (long long)ny * (iz + 1));
    T3[node] = T2i[node] + S * pred[v];
  }
}

inline int ugrid(long long n, int block = 256) {
  long long g = (n + block - 1) / block;
  if (g > 152 * 32) g = 152 * 32;
  return g < 1 ? 1 : (int)g;
}

}  // namespace gm

using namespace gm;

static Grid5 grid5(const int g[4]) { return Grid5{g[0], g[1], g[2], g[3]}; }

// The warp-level (mma.sync) form of the convolution: any slice alignment,
// Cout in {16, 32, 64, 96, 128, 192}.
extern "C" int gm_unet_conv3_mma(const gm_conv_args* c, void* stream) {
  if (!c || !c->in || !c->w || !c->out) return GM_ERR_ARG;
  if (c->cin < 16 || c->cin % 16 || c->cin + c->in_off > c->in_stride || c->cout + c->out_off > c->out_stride)
    return GM_ERR_ARG;
  if (c->in_off % 2 || c->in_stride % 2 || c->out_off % 2 || c->out_stride % 2) return GM_ERR_ARG;
  if (c->mask && (c->mask_off % 2 || c->mask_stride % 2 || c->cout + c->mask_off > c->mask_stride)) return GM_ERR_ARG;
  for (int d = 0; d < 4; ++d)
    if (c->grid[d] < 1) return GM_ERR_ARG;
  if (c->grid[1] > 1023 || c->grid[2] > 1023 || c->grid[3] > 1023) return GM_ERR_TOO_LARGE;
  if ((long long)c->grid[0] * c->grid[1] * c->grid[2] * c->grid[3] >= (1LL << 31)) return GM_ERR_TOO_LARGE;
  ConvK a;
  a.g = grid5(c->grid);
  a.cin = c->cin;
  a.in_stride = c->in_stride;
  a.in_off = c->in_off;
  a.out_stride = c->out_stride;
  a.out_off = c->out_off;
  a.mask_stride = c->mask_stride;
  a.mask_off = c->mask_off;
  a.mirror = c->mirror;
  a.relu = c->relu;
  a.in = (const uint16_t*)c->in;
  a.w = (const uint16_t*)c->w;
  a.bias = c->bias;
  a.mask = (const uint16_t*)c->mask;
  a.out = (uint16_t*)c->out;
  const long long V = (long long)a.g.B * a.g.X * a.g.Y * a.g.Z;
  const size_t smem = (size_t)c->cout * (c->cin + 8) * 2;
  cudaStream_t st = (cudaStream_t)stream;
#define GM_CONV_CASE(N)                                                                                   \
  case N: {                                                                                               \
    const long long rows = (long long)CV_WARPS * ConvShape<N>::ROWS;                                      \
    if (smem > 48 * 1024 &&                                                                               \
        cudaFuncSetAttribute(conv3_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != \
            cudaSuccess)                                                                                  \
      return GM_ERR_LAUNCH;                                                                               \
    conv3_kernel<N><<<(unsigned)((V + rows - 1) / rows), CV_WARPS * 32, smem, st>>>(a);                   \
    break;                                                                                                \
  }
  switch (c->cout) {
    GM_CONV_CASE(16)
    GM_CONV_CASE(32)
    GM_CONV_CASE(64)
    GM_CONV_CASE(96)
    GM_CONV_CASE(128)
    GM_CONV_CASE(192)
    default:
      return GM_ERR_ARG;
  }
#undef GM_CONV_CASE
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_unet_conv3_tc_eligible(const gm_conv_args* c);
extern "C" int gm_unet_conv3_tc(const gm_conv_args* c, void* stream);

// The tensor-core (tcgen05) form where the call allows it, else mma.sync.
extern "C" int gm_unet_conv3(const gm_conv_args* c, void* stream) {
  if (c && gm_unet_conv3_tc_eligible(c)) {
    for (int d = 0; d < 4; ++d)
      if (c->grid[d] < 1) return GM_ERR_ARG;
    return gm_unet_conv3_tc(c, stream);
  }
  return gm_unet_conv3_mma(c, stream);
}

extern "C" long long gm_unet_wgrad_scratch(const int grid[4], int cin, int cout) {
  const long long V = (long long)grid[0] * grid[1] * grid[2] * grid[3];
  long long ns = V / 2048;
  if (ns < 1) ns = 1;
  if (ns > 64) ns = 64;
  return ns * 27 * (long long)cin * cout;
}

extern "C" int gm_unet_wgrad(const gm_wgrad_args* c, void* stream) {
  if (!c || !c->in || !c->dy || !c->dw || !c->scratch) return GM_ERR_ARG;
  if ((c->cin % 32 && c->cin != 16) || c->cout % 16 || c->cout < 16) return GM_ERR_ARG;
  const int nb8 = c->cin >= 32 ? 4 : 2;
  if ((c->cout / 16) * (c->cin / (nb8 * 8)) > 4 * WG_WARPS) return GM_ERR_ARG;
  if (c->in_off % 2 || c->in_stride % 2 || c->dy_off % 2 || c->dy_stride % 2) return GM_ERR_ARG;
  const long long need = gm_unet_wgrad_scratch(c->grid, c->cin, c->cout);
  if (need > c->scratch_cap) return GM_ERR_TOO_LARGE;
  WgradK a;
  a.g = grid5(c->grid);
  a.cin = c->cin;
  a.cout = c->cout;
  a.in_stride = c->in_stride;
  a.in_off = c->in_off;
  a.dy_stride = c->dy_stride;
  a.dy_off = c->dy_off;
  a.in = (const uint16_t*)c->in;
  a.dy = (const uint16_t*)c->dy;
  a.part = c->scratch;
  const long long V = (long long)a.g.B * a.g.X * a.g.Y * a.g.Z;
  a.nsplit = (int)(need / (27LL * c->cin * c->cout));
  a.chunk = (V + a.nsplit - 1) / a.nsplit;
  a.chunk = (a.chunk + WG_KV - 1) / WG_KV * WG_KV;
  const size_t smem = (size_t)WG_KV * ((c->cout + 8) + (c->cin + 8)) * 2;
  cudaStream_t st = (cudaStream_t)stream;
  if (smem > 48 * 1024 &&
      (cudaFuncSetAttribute(wgrad_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
       cudaFuncSetAttribute(wgrad_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess))
    return GM_ERR_LAUNCH;
  if (nb8 == 4)
    wgrad_kernel<4><<<dim3(a.nsplit, 27), WG_WARPS * 32, smem, st>>>(a);
  else
    wgrad_kernel<2><<<dim3(a.nsplit, 27), WG_WARPS * 32, smem, st>>>(a);
  if (cudaGetLastError() != cudaSuccess) return GM_ERR_LAUNCH;
  const long long n = 27LL * c->cin * c->cout;
  sum_splits_kernel<<<ugrid(n), 256, 0, st>>>(c->scratch, a.nsplit, n, c->dw, 1.0f);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_unet_bias_grad(const int grid[4], int C, const void* dy, int stride, int off, float* scratch,
                                 long long scratch_cap, float* db, void* stream) {
  if (!grid || !dy || !scratch || !db || C < 1) return GM_ERR_ARG;
  const long long V = (long long)grid[0] * grid[1] * grid[2] * grid[3];
  long long nb = (V + 4095) / 4096;
  if (nb > 1024) nb = 1024;
  const long long chunk = (V + nb - 1) / nb;
  if (nb * C > scratch_cap) return GM_ERR_TOO_LARGE;
  cudaStream_t st = (cudaStream_t)stream;
  bias_grad_kernel<<<(unsigned)nb, 128, 0, st>>>(V, C, (const uint16_t*)dy, stride, off, chunk, scratch);
  if (cudaGetLastError() != cudaSuccess) return GM_ERR_LAUNCH;
  sum_splits_kernel<<<ugrid(C), 256, 0, st>>>(scratch, (int)nb, C, db, 1.0f);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_unet_pool2(const int grid[4], int C, const void* in, int is, int io, void* out, int os, int oo,
                             int backward, void* stream) {
  if (!grid || !in || !out || C < 1 || grid[1] % 2 || grid[2] % 2 || grid[3] % 2) return GM_ERR_ARG;
  const long long n = (long long)grid[0] * grid[1] * grid[2] * grid[3] * C;
  if (vec8_ok(grid, C, in, is, io, out, os, oo)) {  // 8 channels a thread
    resample8_kernel<<<ugrid(n / 8), 256, 0, (cudaStream_t)stream>>>(grid5(grid), C / 8, (const uint16_t*)in, is, io,
                                                                     (uint16_t*)out, os, oo, !backward, 0.125f, 0);
    return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
  }
  pool2_kernel<<<ugrid(n), 256, 0, (cudaStream_t)stream>>>(grid5(grid), C, (const uint16_t*)in, is, io,
                                                           (uint16_t*)out, os, oo, backward);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_unet_up2(const int grid[4], int C, const void* in, int is, int io, void* out, int os, int oo,
                           int backward, void* stream) {
  if (!grid || !in || !out || C < 1 || grid[1] % 2 || grid[2] % 2 || grid[3] % 2) return GM_ERR_ARG;
  const long long n = (long long)grid[0] * grid[1] * grid[2] * grid[3] * C;
  if (vec8_ok(grid, C, in, is, io, out, os, oo)) {  // 8 channels a thread
    resample8_kernel<<<ugrid(n / 8), 256, 0, (cudaStream_t)stream>>>(grid5(grid), C / 8, (const uint16_t*)in, is, io,
                                                                     (uint16_t*)out, os, oo, backward, 1.f, !backward);
    return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
  }
  up2_kernel<<<ugrid(n), 256, 0, (cudaStream_t)stream>>>(grid5(grid), C, (const uint16_t*)in, is, io,
                                                         (uint16_t*)out, os, oo, backward);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_unet_add_slice(long long V, int C, const void* a, int as, int ao, void* b, int bs, int bo,
                                 const void* mask, int ms, int mo, void* stream) {
  if (!a || !b || V < 0 || C < 1) return GM_ERR_ARG;
  add_slice_kernel<<<ugrid(V * C), 256, 0, (cudaStream_t)stream>>>(V, C, (const uint16_t*)a, as, ao, (uint16_t*)b,
                                                                   bs, bo, (const uint16_t*)mask, ms, mo);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_unet_head(long long V, int C, const void* in, int is, int io, const float* w, float b, float* out,
                            void* stream) {
  if (!in || !w || !out || V < 0 || C < 1) return GM_ERR_ARG;
  head_fwd_kernel<<<ugrid(V), 256, 0, (cudaStream_t)stream>>>(V, C, (const uint16_t*)in, is, io, w, b, out);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" long long gm_unet_head_scratch(long long V, int C) {
  long long nb = (V + 8191) / 8192;
  if (nb < 1) nb = 1;
  return nb * (C + 2);
}

extern "C" int gm_unet_head_bwd(long long V, int C, const void* in, int is, int io, const float* w, const float* pred,
                                const float* target, const float* lmask, float inv_count, void* din, int ds, int dof,
                                float* scratch, long long scratch_cap, float* dwb, void* stream) {
  if (!in || !w || !pred || !target || !din || !scratch || !dwb || V < 1 || C < 1) return GM_ERR_ARG;
  const long long need = gm_unet_head_scratch(V, C);
  if (need > scratch_cap) return GM_ERR_TOO_LARGE;
  const long long nb = need / (C + 2);
  const long long chunk = (V + nb - 1) / nb;
  cudaStream_t st = (cudaStream_t)stream;
  if (C > HB_CMAX) return GM_ERR_ARG;
  head_bwd_kernel<<<(unsigned)nb, HB_THREADS, 0, st>>>(V, C, (const uint16_t*)in, is, io, w, pred, target, lmask,
                                                       inv_count, (uint16_t*)din, ds, dof, chunk, scratch);
  if (cudaGetLastError() != cudaSuccess) return GM_ERR_LAUNCH;
  sum_splits_kernel<<<ugrid(C + 2), 256, 0, st>>>(scratch, (int)nb, C + 2, dwb, 1.0f);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_unet_adam(const gm_adam_args* c, void* stream) {
  if (!c || !c->w || !c->grad || !c->m || !c->v || c->n < 0) return GM_ERR_ARG;
  if (c->wt && (!c->wb || c->cout < 1 || c->cin < 1 || c->n % ((long long)c->cout * c->cin))) return GM_ERR_ARG;
  adam_kernel<<<ugrid(c->n), 256, 0, (cudaStream_t)stream>>>(c->n, c->w, c->grad, c->m, c->v, c->lr, c->beta1,
                                                            c->beta2, c->eps, c->c1, c->c2, c->wd,
                                                            (uint16_t*)c->wb, (uint16_t*)c->wt, c->cout, c->cin);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_surrogate_pack(const gm_surr_args* c, void* stream) {
  if (!c || !c->T2i || !c->T3o || !c->par || !c->x) return GM_ERR_ARG;
  if (c->grid[1] > c->nodes[0] || c->grid[2] > c->nodes[1] || c->grid[3] + 1 > c->nodes[2] || c->grid[0] < 1)
    return GM_ERR_ARG;
  const long long V = (long long)c->grid[0] * c->grid[1] * c->grid[2] * c->grid[3];
  const long long nn = (long long)c->nodes[0] * c->nodes[1] * c->nodes[2];
  surr_pack_kernel<<<ugrid(V), 256, 0, (cudaStream_t)stream>>>(grid5(c->grid), c->nodes[0], c->nodes[1], nn, c->T2i,
                                                               c->T3o, c->T3n, c->par, (float)c->T_amb,
                                                               (float)c->scale, (uint16_t*)c->x, c->target, c->lmask);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

extern "C" int gm_surrogate_unpack(const gm_surr_args* c, const float* pred, float* T3, void* stream) {
  if (!c || !c->T2i || !pred || !T3) return GM_ERR_ARG;
  if (c->grid[1] > c->nodes[0] || c->grid[2] > c->nodes[1] || c->grid[3] + 1 > c->nodes[2] || c->grid[0] < 1)
    return GM_ERR_ARG;
  const long long V = (long long)c->grid[0] * c->grid[1] * c->grid[2] * c->grid[3];
  const long long nn = (long long)c->nodes[0] * c->nodes[1] * c->nodes[2];
  surr_unpack_kernel<<<ugrid(V), 256, 0, (cudaStream_t)stream>>>(grid5(c->grid), c->nodes[0], c->nodes[1], nn,
                                                                 c->T2i, pred, (float)c->scale, T3);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}
