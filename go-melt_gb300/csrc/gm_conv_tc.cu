// 3x3x3 convolution of the Level-3 surrogate on the Blackwell tensor cores
// (tcgen05.mma, BF16 in, FP32 accumulate in tensor memory).  No counterpart
// in the reference.
//
// Implicit GEMM: M = voxels (a tile of 16 x 8 voxels of one z plane and one
// sample = 128 rows), N = output channels, K = 27 taps x input channels.
// Per tap, the A tile is the input box shifted by the tap offset and the B
// tile the tap's weights; both are brought into shared memory by TMA
// (cp.async.bulk.tensor) in 8-channel column blocks, which is exactly the
// K-major no-swizzle canonical layout of the MMA operands: within a column
// block rows are 16 bytes apart, so 8-row core matrices are contiguous
// (stride-dimension offset 128 B) and column blocks follow each other
// (leading-dimension offset = one block).  The TMA box of the input starts at
// the shifted voxel coordinates; parts outside the sample are filled with
// zeros by the copy engine, which is the convolution's zero padding.
//
// One thread issues the copies and the MMAs through a ring of `stages`
// shared-memory stages (full / empty mbarriers: a stage is refilled once the
// MMAs reading it have completed, tcgen05.commit).  After the last tap the
// four warps read the 128 x N accumulator from tensor memory (each warp its 32
// lanes = rows), add the bias, apply ReLU and the mask, and store BF16.
//
// Waits are bounded (about one second): on a timeout the CTA records it in a
// status word, lets outstanding copies and MMAs finish (again bounded),
// frees its tensor memory and returns without writing.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "gm_common.cuh"

namespace gm {

constexpr int TC_BX = 16, TC_BY = 8;  // voxel box of an M tile: 128 rows, row = x + 16 y
constexpr int TC_MAX_STAGES = 4;
constexpr long long TC_WAIT_CYCLES = 2000000000LL;

__device__ int g_tc_status;  // bit 0: a wait ran out

struct ConvTC {
  int X, Y, Z, B;
  int cin, cout, mirror, relu, stages;
  unsigned ncols;  // tensor-memory columns allocated (power of two >= 32)
  int out_stride, out_off, mask_stride, mask_off;
  const float* bias;
  const uint16_t* mask;
  uint16_t* out;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.b32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase of `parity` to complete; false on a timeout.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_test(bar, parity))
    if (clock64() - t0 > TC_WAIT_CYCLES) return false;
  return true;
}

__device__ __forceinline__ void tma_load_5d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            int c4, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], "
      "[%7];" ::"r"(dst),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(map), "r"(c0), "r"(c1), "r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor: K-major, no swizzle; lbo = byte offset
// between core matrices adjacent along K, sbo = along M/N.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M x N.
__host__ __device__ constexpr uint32_t mma_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
          tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack2_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

__global__ void __launch_bounds__(128, 1)
    conv3_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, const ConvTC a) {
  extern __shared__ __align__(1024) uint8_t smraw[];
  __shared__ __align__(8) uint64_t bar_full[TC_MAX_STAGES], bar_empty[TC_MAX_STAGES], bar_done;
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int tiles_x = (a.X + TC_BX - 1) / TC_BX, tiles_y = (a.Y + TC_BY - 1) / TC_BY;
  int t = blockIdx.x;
  const int tx = t % tiles_x;
  t /= tiles_x;
  const int ty = t % tiles_y;
  t /= tiles_y;
  const int z0 = t % a.Z, bs = t / a.Z;
  const int x0 = tx * TC_BX, y0 = ty * TC_BY;
  const int kg = a.cin / 8;
  const uint32_t a_bytes = (uint32_t)kg * 128u * 16u, blk_b = (uint32_t)a.cout * 16u;
  const uint32_t stage_bytes = a_bytes + (uint32_t)kg * blk_b;
  // 1024-byte aligned start of the stages in the dynamic window
  const uint32_t base = (smem_u32(smraw) + 1023u) & ~1023u;
  const int S = a.stages;

  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(smem_u32(&bar_full[s]), 1);
      mbar_init(smem_u32(&bar_empty[s]), 1);
    }
    mbar_init(smem_u32(&bar_done), 1);
    s_fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(a.ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  if (tid == 0) {
    const uint32_t idesc = mma_idesc(128, a.cout);
    int loaded = 0;  // taps whose copies were issued
    auto load = [&](int tap) {
      const int s = tap % S;
      int dx = tap % 3 - 1, dy = (tap / 3) % 3 - 1, dz = tap / 9 - 1;
      if (a.mirror) {
        dx = -dx;
        dy = -dy;
        dz = -dz;
      }
      const uint32_t st = base + (uint32_t)s * stage_bytes, bar = smem_u32(&bar_full[s]);
      mbar_expect_tx(bar, stage_bytes);
      for (int j = 0; j < kg; ++j) tma_load_5d(st + (uint32_t)j * 2048u, &tmA, 8 * j, x0 + dx, y0 + dy, z0 + dz, bs, bar);
      for (int j = 0; j < kg; ++j) tma_load_2d(st + a_bytes + (uint32_t)j * blk_b, &tmB, 8 * j, tap * a.cout, bar);
      loaded = tap + 1;
    };
    for (int tap = 0; tap < S && tap < 27; ++tap) load(tap);
    bool ok = true;
    int consumed = 0;
    for (int tap = 0; tap < 27 && ok; ++tap) {
      const int s = tap % S;
      const uint32_t par = (uint32_t)(tap / S) & 1u;
      if (!mbar_wait(smem_u32(&bar_full[s]), par)) {
        ok = false;
        break;
      }
      consumed = tap + 1;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t st = base + (uint32_t)s * stage_bytes;
      for (int k = 0; k < kg / 2; ++k) {  // 16 channels an MMA
        const uint64_t ad = smem_desc(st + (uint32_t)(2 * k) * 2048u, 2048u, 128u);
        const uint64_t bd = smem_desc(st + a_bytes + (uint32_t)(2 * k) * blk_b, blk_b, 128u);
        mma_bf16(tmem, ad, bd, idesc, (tap > 0 || k > 0) ? 1u : 0u);
      }
      mma_commit(smem_u32(&bar_empty[s]));
      if (tap + S < 27) {
        if (!mbar_wait(smem_u32(&bar_empty[s]), par)) {  // the MMAs reading stage s are done
          ok = false;
          break;
        }
        load(tap + S);
      }
    }
    if (!ok) {
      s_fail = 1;
      atomicOr(&g_tc_status, 1);
      // let the copies already issued land before the CTA leaves (bounded)
      for (int tap = consumed; tap < loaded; ++tap)
        mbar_wait(smem_u32(&bar_full[tap % S]), (uint32_t)(tap / S) & 1u);
    }
    mma_commit(smem_u32(&bar_done));  // arrives once every MMA issued above has completed
  }
  __syncwarp();
  const bool done = mbar_wait(smem_u32(&bar_done), 0);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  __syncthreads();
  if (!done && tid == 0) atomicOr(&g_tc_status, 1);
  if (done && !s_fail) {
    // epilogue: row r = tid <-> voxel (x0 + r % 16, y0 + r / 16, z0, bs)
    const int x = x0 + (tid & 15), y = y0 + (tid >> 4);
    const bool live = x < a.X && y < a.Y;
    const long long v = (((long long)bs * a.Z + z0) * a.Y + y) * a.X + x;
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    for (int c = 0; c < a.cout; c += 8) {
      float f[8];
      tmem_ld8(trow + (uint32_t)c, f);
      if (!live) continue;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        if (a.bias) f[i] += a.bias[c + i];
        if (a.relu) f[i] = fmaxf(f[i], 0.f);
        if (a.mask) {
          const uint16_t m = a.mask[v * a.mask_stride + a.mask_off + c + i];
          if (!(__uint_as_float((uint32_t)m << 16) > 0.f)) f[i] = 0.f;
        }
      }
      uint16_t* o = a.out + v * a.out_stride + a.out_off + c;
      const uint4 pk = make_uint4(pack2_bf16(f[0], f[1]), pack2_bf16(f[2], f[3]), pack2_bf16(f[4], f[5]),
                                  pack2_bf16(f[6], f[7]));
      *reinterpret_cast<uint4*>(o) = pk;  // 16-byte aligned: out_stride, out_off multiples of 8
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(a.ncols) : "memory");
}

}  // namespace gm

using namespace gm;

namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled from the driver, looked up once (no link-time
// dependency on libcuda).
EncodeTiledFn encode_fn() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
    else
      cudaGetLastError();
  });
  return fn;
}

size_t smem_optin() {
  static size_t cap = 0;
  if (cap == 0) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cap = v > 0 ? (size_t)v : 232448;
  }
  return cap;
}

}  // namespace

// Whether the tensor-core path takes a convolution: channel counts multiples
// of 16 (Cout <= 256), 16-byte aligned slices and bases (TMA, vector stores).
extern "C" int gm_unet_conv3_tc_eligible(const gm_conv_args* c) {
  if (!c || !c->in || !c->w || !c->out) return 0;
  if (c->cin < 16 || c->cin % 16 || c->cout < 16 || c->cout % 16 || c->cout > 256) return 0;
  if (c->in_off % 8 || c->in_stride % 8 || c->out_off % 8 || c->out_stride % 8) return 0;
  if (((uintptr_t)c->in | (uintptr_t)c->w | (uintptr_t)c->out) & 15) return 0;
  if (c->cin + c->in_off > c->in_stride || c->cout + c->out_off > c->out_stride) return 0;
  if (c->mask && c->cout + c->mask_off > c->mask_stride) return 0;
  const size_t stage = (size_t)(c->cin / 8) * 128 * 16 + (size_t)(c->cin / 8) * c->cout * 16;
  if (stage + 1024 > smem_optin() - 1024) return 0;
  return encode_fn() != nullptr;
}

extern "C" int gm_unet_conv3_tc(const gm_conv_args* c, void* stream) {
  if (!c) return GM_ERR_ARG;
  for (int d = 0; d < 4; ++d)
    if (c->grid[d] < 1) return GM_ERR_ARG;
  if (!gm_unet_conv3_tc_eligible(c)) return GM_ERR_UNSUPPORTED;
  const int B = c->grid[0], X = c->grid[1], Y = c->grid[2], Z = c->grid[3];
  const long long tiles = (long long)((X + TC_BX - 1) / TC_BX) * ((Y + TC_BY - 1) / TC_BY) * Z * B;
  if (tiles >= (1LL << 31) || (long long)B * X * Y * Z >= (1LL << 31)) return GM_ERR_TOO_LARGE;
  EncodeTiledFn enc = encode_fn();
  CUtensorMap ta, tb;
  // input slice as a 5-D tensor {channels, x, y, z, sample}, zero fill outside
  const cuuint64_t vb = (cuuint64_t)c->in_stride * 2;
  const cuuint64_t dimA[5] = {(cuuint64_t)c->cin, (cuuint64_t)X, (cuuint64_t)Y, (cuuint64_t)Z, (cuuint64_t)B};
  const cuuint64_t strA[4] = {vb, vb * X, vb * X * Y, vb * X * Y * Z};
  const cuuint32_t boxA[5] = {8, TC_BX, TC_BY, 1, 1};
  const cuuint32_t one[5] = {1, 1, 1, 1, 1};
  if (enc(&ta, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, (void*)((const uint16_t*)c->in + c->in_off), dimA, strA, boxA, one,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return GM_ERR_UNSUPPORTED;
  // weights [27 * cout rows][cin]
  const cuuint64_t dimB[2] = {(cuuint64_t)c->cin, (cuuint64_t)27 * c->cout};
  const cuuint64_t strB[1] = {(cuuint64_t)c->cin * 2};
  const cuuint32_t boxB[2] = {8, (cuuint32_t)c->cout};
  if (enc(&tb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)c->w, dimB, strB, boxB, one, CU_TENSOR_MAP_INTERLEAVE_NONE,
          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
      CUDA_SUCCESS)
    return GM_ERR_UNSUPPORTED;
  ConvTC a;
  a.X = X;
  a.Y = Y;
  a.Z = Z;
  a.B = B;
  a.cin = c->cin;
  a.cout = c->cout;
  a.mirror = c->mirror;
  a.relu = c->relu;
  const size_t stage = (size_t)(c->cin / 8) * 128 * 16 + (size_t)(c->cin / 8) * c->cout * 16;
  const size_t cap = smem_optin() - 1024;  // less the static shared memory and the alignment pad
  int S = (int)((cap - 1024) / stage);
  a.stages = S > TC_MAX_STAGES ? TC_MAX_STAGES : S;
  unsigned nc = 32;
  while (nc < (unsigned)c->cout) nc <<= 1;
  a.ncols = nc;
  a.out_stride = c->out_stride;
  a.out_off = c->out_off;
  a.mask_stride = c->mask_stride;
  a.mask_off = c->mask_off;
  a.bias = c->bias;
  a.mask = (const uint16_t*)c->mask;
  a.out = (uint16_t*)c->out;
  const size_t smem = (size_t)a.stages * stage + 1024;
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    attr = cudaFuncSetAttribute(conv3_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(smem_optin() - 1024));
  });
  if (attr != cudaSuccess) return GM_ERR_LAUNCH;
  conv3_tc_kernel<<<(unsigned)tiles, 128, smem, (cudaStream_t)stream>>>(ta, tb, a);
  return cudaGetLastError() == cudaSuccess ? GM_OK : GM_ERR_LAUNCH;
}

// Status of the tensor-core convolutions since the last call (bit 0: a wait
// ran out); the word is cleared.  Synchronises the device.
extern "C" int gm_unet_tc_status(void) {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_tc_status, sizeof(int)) != cudaSuccess) return -1;
  const int zero = 0;
  cudaMemcpyToSymbol(g_tc_status, &zero, sizeof(int));
  return v;
}
