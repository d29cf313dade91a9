// 3x3x3 convolution of the Level-3 surrogate on the Blackwell tensor cores
// (tcgen05.mma, BF16 in, FP32 accumulate in tensor memory).  No counterpart
// in the reference.
//
// Implicit GEMM: M = voxels (a tile of 8 x 16 voxels of one z plane and one
// sample = 128 rows, row = x + 8 y), N = output channels, K = 27 taps x input
// channels.  Per chunk of input channels the CTA's threads load the tile's
// halo box of 10 x 18 x 3 voxels into shared memory once (16-byte vectors,
// zeros outside the sample: the convolution's zero padding) in the K-major
// no-swizzle canonical layout of the MMA operands: one 8-channel block after
// the other, within a block a voxel is a 16-byte row, x fastest, so 8
// consecutive x voxels form a contiguous 8-row core matrix and the core
// matrices of the tile's y rows lie 10 voxels (160 bytes, the
// stride-dimension offset) apart.  The A operand of tap (dx, dy, dz) is then
// the same box addressed from the voxel offset ((dz * 18 + dy) * 10 + dx):
// all 27 taps read one copy of the input.  (A tensor copy of this box moves
// 16-byte rows, one per voxel and block, at about 0.1 row a cycle and SM --
// measured -- which bound every full-resolution layer; the threads' vector
// loads are coalesced over the voxel records.)  B is the tap's weights for
// the chunk: 8-channel column blocks of cout 16-byte rows, one contiguous bulk
// copy per tile from a per-call prepacked copy of the weights (wpack), or a
// tensor copy per block from the [27][cout][cin] weights.
//
// Thread 0 issues the weight copies and the MMAs: the halo boxes of two
// chunks in two buffers, the (chunk, tap) weight tiles through a ring of
// `stages` shared-memory stages (full / empty mbarriers; a stage is refilled
// once the MMAs reading it have completed, tcgen05.commit, checked one tap
// late so that the next tap's MMAs are queued behind the running ones and the
// tensor pipe does not drain between taps).  After the last tap the four
// warps read the 128 x N accumulator from tensor memory (each warp its 32
// lanes = rows), add the bias, apply ReLU and the mask, and store BF16.
//
// Waits are bounded (about one second): on a timeout the CTA records it in a
// status word, lets outstanding copies and MMAs finish (again bounded),
// frees its tensor memory and returns without writing.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <stdlib.h>

#include <initializer_list>
#include <mutex>

#include "gm_common.cuh"

namespace gm {

constexpr int TC_BX = 8, TC_BY = 16;        // voxel box of an M tile: 128 rows, row = x + 8 y
constexpr int TC_HX = TC_BX + 2, TC_HY = TC_BY + 2, TC_HZ = 3;  // its halo box
constexpr uint32_t TC_HALO_BYTES = TC_HX * TC_HY * TC_HZ * 16;   // one 8-channel block of the halo (8640)
constexpr uint32_t TC_HALO_STRIDE = (TC_HALO_BYTES + 127) / 128 * 128;  // blocks 128-byte aligned (8704)
constexpr int TC_MAX_STAGES = 32;                // weight stages (every tap of a chunk where they fit)
constexpr size_t TC_SMEM_TARGET = 112 * 1024;   // stage budget: two CTAs an SM
constexpr long long TC_WAIT_CYCLES = 2000000000LL;

__device__ int g_tc_status;  // bit 0: a wait ran out

struct ConvTC {
  const uint16_t* in;     // input slice base (element in_off of voxel 0)
  int in_stride;          // elements a voxel
  const uint16_t* wpack;  // weights in the tile layout [chunk][tap][block][cout][8], or NULL
  int X, Y, Z, B;
  int cin, cout, mirror, relu, stages;
  int cc;          // input channels a chunk (a multiple of 16 dividing cin)
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

// One contiguous bulk copy (no tensor map) into shared memory, completing on `bar`.
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
// Bounded wait of warps with nothing else to do: polls with a short sleep so
// that the issuing warps keep the schedulers.
__device__ __forceinline__ bool mbar_wait_idle(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_test(bar, parity)) {
    if (clock64() - t0 > TC_WAIT_CYCLES) return false;
    __nanosleep(64);
  }
  return true;
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
// One lane of the (converged) warp: true there, false elsewhere.
__device__ __forceinline__ bool elect_one() {
  uint32_t p = 0;
  asm volatile("{\n .reg .pred P;\n elect.sync _|P, 0xffffffff;\n selp.b32 %0, 1, 0, P;\n}" : "=r"(p));
  return p != 0;
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
    conv3_tc_kernel(const __grid_constant__ CUtensorMap tmB, const ConvTC a) {
  extern __shared__ __align__(1024) uint8_t smraw[];
  __shared__ __align__(8) uint64_t bar_full[TC_MAX_STAGES], bar_empty[TC_MAX_STAGES], bar_aempty[2], bar_done;
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
  const int cb = a.cc / 8;                    // 8-channel blocks a chunk
  const int nch = a.cin / a.cc;               // chunks
  const int nA = nch > 1 ? 2 : 1;             // halo buffers
  const int total = 27 * nch;                 // (chunk, tap) steps
  const uint32_t a_bytes = (uint32_t)cb * TC_HALO_STRIDE;
  const uint32_t blk_b = (uint32_t)a.cout * 16u, stage_bytes = (uint32_t)cb * blk_b;
  // 1024-byte aligned start of the halo buffers, then the weight stages
  const uint32_t base = (smem_u32(smraw) + 1023u) & ~1023u;
  const uint32_t bbase = base + (uint32_t)nA * a_bytes;
  const int S = a.stages;

  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(smem_u32(&bar_full[s]), 1);
      mbar_init(smem_u32(&bar_empty[s]), 1);
    }
    for (int s = 0; s < 2; ++s) mbar_init(smem_u32(&bar_aempty[s]), 1);
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

  const uint32_t idesc = mma_idesc(128, a.cout);
  // One warp issues (warp blockIdx % 4, so that the CTAs resident on an SM
  // issue from different schedulers): its lanes run the loops below
  // converged (the addresses and descriptors stay warp-uniform) and one lane,
  // chosen by elect.sync, issues each copy, MMA and commit.
  const bool issuer = warp == (int)(blockIdx.x & 3);  // CTAs on one SM issue from different schedulers
  const bool leader = issuer && elect_one();
  int issuedB = 0, waitedB = 0;  // weight copies issued / waited for (for the drain)
  auto loadB = [&](int idx) {    // weights of tap idx % 27 for chunk idx / 27
    const int c = idx / 27, tap = idx % 27, s = idx % S;
    const uint32_t dst = bbase + (uint32_t)s * stage_bytes, bar = smem_u32(&bar_full[s]);
    if (leader) {
      mbar_expect_tx(bar, stage_bytes);
      if (a.wpack)  // the tile, prepacked: [block][cout][8] contiguous
        bulk_load(dst, a.wpack + (size_t)(c * 27 + tap) * cb * a.cout * 8, stage_bytes, bar);
      else
        for (int j = 0; j < cb; ++j) tma_load_2d(dst + (uint32_t)j * blk_b, &tmB, c * a.cc + 8 * j, tap * a.cout, bar);
    }
    issuedB = idx + 1;
  };
  // every weight tile resident (S >= total) and prepacked: one bulk copy for all
  // of them (a copy costs the SM's copy engine about as much as a tile's MMAs,
  // so 27 copies a tile would bound the kernel), completing on bar_full[0]
  const bool one_copy = a.wpack && S >= total;
  if (issuer) {
    if (one_copy) {
      if (leader) {
        mbar_expect_tx(smem_u32(&bar_full[0]), (uint32_t)total * stage_bytes);
        bulk_load(bbase, a.wpack, (uint32_t)total * stage_bytes, smem_u32(&bar_full[0]));
      }
      issuedB = 1;
    } else {
      for (int idx = 0; idx < S && idx < total; ++idx) loadB(idx);
    }
    __syncwarp();
  }

  for (int c = 0; c < nch; ++c) {
    const int buf = c % nA;
    // the buffer's previous chunk (c - 2) must be done with it
    if (c >= 2 && !mbar_wait_idle(smem_u32(&bar_aempty[buf]), (uint32_t)((c - 2) / 2) & 1u)) atomicOr(&s_fail, 1);
    // ---- halo box of chunk c by all threads: a voxel's 16-byte blocks per
    // thread, consecutive voxels on consecutive threads (conflict-free shared
    // stores), zeros outside the sample ----
    const uint32_t hb = base + (uint32_t)buf * a_bytes;
    constexpr int NV = TC_HX * TC_HY * TC_HZ;
    for (int v = tid; v < NV; v += 128) {
      const int hx = v % TC_HX, hy = (v / TC_HX) % TC_HY, hz = v / (TC_HX * TC_HY);
      const int x = x0 - 1 + hx, y = y0 - 1 + hy, z = z0 - 1 + hz;
      const bool inb = x >= 0 && x < a.X && y >= 0 && y < a.Y && z >= 0 && z < a.Z;
      const uint4* src = reinterpret_cast<const uint4*>(
          a.in + ((((long long)bs * a.Z + z) * a.Y + y) * a.X + x) * a.in_stride + c * a.cc);
      uint4 q[8];
#pragma unroll
      for (int j = 0; j < 8; ++j)
        q[j] = (inb && j < cb) ? __ldg(src + j) : make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (j < cb) {
          const uint32_t dst = hb + (uint32_t)j * TC_HALO_STRIDE + (uint32_t)v * 16u;
          asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(dst), "r"(q[j].x), "r"(q[j].y), "r"(q[j].z),
                       "r"(q[j].w)
                       : "memory");
        }
    }
    // the tensor cores read shared memory through the async proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (s_fail) break;
    if (issuer) {
      bool ok = true;
      // descriptors: only the start-address field (bits 0-13, address / 16)
      // changes between taps, k-steps and stages
      const uint64_t ad0 = smem_desc(hb, TC_HALO_STRIDE, TC_HX * 16u);
      const uint64_t bd0 = smem_desc(bbase, blk_b, 128u);
      const uint32_t a_k = 2u * TC_HALO_STRIDE / 16u, b_k = 2u * blk_b / 16u, b_s = stage_bytes / 16u;
      int s = (c * 27) % S, ph = ((c * 27) / S) & 1;  // stage and parity of step (c, 0)
#pragma unroll 3
      for (int tap = 0; tap < 27 && ok; ++tap) {
        const int idx = c * 27 + tap;
        const bool got = one_copy ? (idx > 0 || mbar_wait(smem_u32(&bar_full[0]), 0u))
                                  : mbar_wait(smem_u32(&bar_full[s]), (uint32_t)ph);
        if (!__all_sync(0xffffffffu, got)) {
          ok = false;
          break;
        }
        waitedB = one_copy ? 1 : idx + 1;
        if (leader) {
          // tap offset within the halo box (mirrored taps, the data gradient: tap 26 - t)
          const int tt = a.mirror ? 26 - tap : tap;
          const uint32_t toff = (uint32_t)(((tt / 9) * TC_HY + (tt / 3) % 3) * TC_HX + tt % 3);  // voxels
          const uint64_t ad = ad0 + toff;  // 16 bytes a voxel row: the address field counts 16-byte units
          const uint64_t bd = bd0 + (uint64_t)s * b_s;
          // order the MMAs after the synchronisation they depend on: the halo
          // barrier (first tap of a chunk) and, for streamed weights, this tap's wait
          if (tap == 0 || !one_copy) asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          for (int k = 0; k < cb / 2; ++k)  // 16 channels an MMA
            mma_bf16(tmem, ad + (uint64_t)k * a_k, bd + (uint64_t)k * b_k, idesc, (idx > 0 || k > 0) ? 1u : 0u);
          if (!one_copy) mma_commit(smem_u32(&bar_empty[s]));
          if (tap == 26 && nA == 2) mma_commit(smem_u32(&bar_aempty[buf]));  // chunk c's MMAs done: buffer free
        }
        if (++s == S) {
          s = 0;
          ph ^= 1;
        }
        __syncwarp();
        // refill the stage of the previous step (its MMAs are queued ahead of this step's)
        if (idx >= 1 && idx - 1 + S < total) {
          const int pidx = idx - 1;
          if (!__all_sync(0xffffffffu, mbar_wait(smem_u32(&bar_empty[pidx % S]), (uint32_t)(pidx / S) & 1u))) {
            ok = false;
            break;
          }
          loadB(pidx + S);
          __syncwarp();
        }
      }
      if (!ok && leader) atomicOr(&s_fail, 1);
    }
  }
  __syncthreads();
  if (issuer) {
    if (s_fail) {
      if (leader) atomicOr(&g_tc_status, 1);
      // let the copies already issued land before the CTA leaves (bounded)
      if (one_copy) {
        if (waitedB < issuedB) mbar_wait(smem_u32(&bar_full[0]), 0u);
      } else {
        for (int i = waitedB; i < issuedB; ++i) mbar_wait(smem_u32(&bar_full[i % S]), (uint32_t)(i / S) & 1u);
      }
    }
    if (leader) mma_commit(smem_u32(&bar_done));  // arrives once every MMA issued above has completed
    __syncwarp();
  }
  __syncwarp();
  const bool done = mbar_wait_idle(smem_u32(&bar_done), 0);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  __syncthreads();
  if (!done && tid == 0) atomicOr(&g_tc_status, 1);
  if (done && !s_fail) {
    // epilogue: row r = tid <-> voxel (x0 + r % 8, y0 + r / 8, z0, bs)
    const int x = x0 + (tid & 7), y = y0 + (tid >> 3);
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

// Weights [27][cout][cin] -> the kernel's weight tiles [chunk][tap][block][cout][8]
// (16-byte vectors: v = ((chunk * 27 + tap) * blocks + block) * cout + n).
__global__ void wpack_kernel(const uint4* __restrict__ w, uint4* __restrict__ p, int cin, int cout, int cc) {
  const int cb = cc / 8;
  const long long nvec = 27LL * cin * cout / 8;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvec; v += (long long)gridDim.x * blockDim.x) {
    const int n = (int)(v % cout);
    long long r = v / cout;
    const int j = (int)(r % cb);
    r /= cb;
    const int tap = (int)(r % 27), c = (int)(r / 27);
    p[v] = w[((long long)tap * cout + n) * (cin / 8) + c * cb + j];
  }
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

// Input channels a chunk: the largest of 64, 48, 32, 16 dividing cin and not
// above GOMELT_CONV_TC_CC when that is set (a tuning override).
int chunk_channels(int cin) {
  static const int cmax = [] {
    const char* e = getenv("GOMELT_CONV_TC_CC");
    const int v = e ? atoi(e) : 0;
    return v >= 16 ? v : 64;
  }();
  for (int cc : {64, 48, 32, 16})
    if (cc <= cmax && cin % cc == 0) return cc;
  return 0;
}

// Shared memory of a launch with `stages` weight stages (halo buffers first).
size_t conv_smem(int cin, int cout, int stages) {
  const int cc = chunk_channels(cin);
  const size_t halo = (size_t)(cin > cc ? 2 : 1) * (cc / 8) * TC_HALO_STRIDE;
  return halo + (size_t)stages * (cc / 8) * cout * 16 + 1024;  // + the 1024-byte alignment pad
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
// of 16 (Cout <= 256), 16-byte aligned slices and bases (vector loads and
// stores, weight copies).
extern "C" int gm_unet_conv3_tc_eligible(const gm_conv_args* c) {
  if (!c || !c->in || !c->w || !c->out) return 0;
  if (c->cin < 16 || c->cin % 16 || c->cout < 16 || c->cout % 16 || c->cout > 256) return 0;
  if (c->in_off % 8 || c->in_stride % 8 || c->out_off % 8 || c->out_stride % 8) return 0;
  if (((uintptr_t)c->in | (uintptr_t)c->w | (uintptr_t)c->out) & 15) return 0;
  if (c->cin + c->in_off > c->in_stride || c->cout + c->out_off > c->out_stride) return 0;
  if (c->mask && c->cout + c->mask_off > c->mask_stride) return 0;
  if (chunk_channels(c->cin) == 0 || conv_smem(c->cin, c->cout, 2) > smem_optin() - 1024) return 0;
  return encode_fn() != nullptr;
}

extern "C" int gm_unet_conv3_tc(const gm_conv_args* c, void* stream) {
  if (!c) return GM_ERR_ARG;
  for (int d = 0; d < 4; ++d)
    if (c->grid[d] < 1) return GM_ERR_ARG;
  if (!gm_unet_conv3_tc_eligible(c)) return GM_ERR_UNSUPPORTED;
  if (c->wpack && (((uintptr_t)c->wpack & 15) || c->wpack == c->w || c->wpack == c->in || c->wpack == c->out))
    return GM_ERR_ARG;
  const int B = c->grid[0], X = c->grid[1], Y = c->grid[2], Z = c->grid[3];
  const long long tiles = (long long)((X + TC_BX - 1) / TC_BX) * ((Y + TC_BY - 1) / TC_BY) * Z * B;
  if (tiles >= (1LL << 31) || (long long)B * X * Y * Z >= (1LL << 31)) return GM_ERR_TOO_LARGE;
  EncodeTiledFn enc = encode_fn();
  CUtensorMap tb;
  const cuuint32_t one[2] = {1, 1};
  // weights [27 * cout rows][cin]
  const cuuint64_t dimB[2] = {(cuuint64_t)c->cin, (cuuint64_t)27 * c->cout};
  const cuuint64_t strB[1] = {(cuuint64_t)c->cin * 2};
  const cuuint32_t boxB[2] = {8, (cuuint32_t)c->cout};
  if (enc(&tb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)c->w, dimB, strB, boxB, one, CU_TENSOR_MAP_INTERLEAVE_NONE,
          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
      CUDA_SUCCESS)
    return GM_ERR_UNSUPPORTED;
  ConvTC a;
  a.in = (const uint16_t*)c->in + c->in_off;
  a.in_stride = c->in_stride;
  a.wpack = (const uint16_t*)c->wpack;
  a.X = X;
  a.Y = Y;
  a.Z = Z;
  a.B = B;
  a.cin = c->cin;
  a.cout = c->cout;
  a.mirror = c->mirror;
  a.relu = c->relu;
  a.cc = chunk_channels(c->cin);
  const size_t cap = smem_optin() - 1024;  // less the static shared memory
  // as many weight stages as the budget holds (at most one per step), at least two
  const int total = 27 * (c->cin / a.cc);
  int S = total < TC_MAX_STAGES ? total : TC_MAX_STAGES;
  // stage budget: TC_SMEM_TARGET, or GOMELT_CONV_TC_SMEM (bytes) when set (a tuning override)
  static const size_t target = [] {
    const char* e = getenv("GOMELT_CONV_TC_SMEM");
    const long long v = e ? atoll(e) : 0;
    return v > 0 ? (size_t)v : TC_SMEM_TARGET;
  }();
  const size_t budget = conv_smem(c->cin, c->cout, 2) > target || target > cap ? cap : target;
  while (S > 2 && conv_smem(c->cin, c->cout, S) > budget) --S;
  a.stages = S;
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
  const size_t smem = conv_smem(c->cin, c->cout, a.stages);
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    attr = cudaFuncSetAttribute(conv3_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(smem_optin() - 1024));
  });
  if (attr != cudaSuccess) return GM_ERR_LAUNCH;
  if (c->wpack) {  // the weight tiles of this call, repacked once
    const long long nvec = 27LL * c->cin * c->cout / 8;
    wpack_kernel<<<(unsigned)((nvec + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        (const uint4*)c->w, (uint4*)c->wpack, c->cin, c->cout, a.cc);
  }
  conv3_tc_kernel<<<(unsigned)tiles, 128, smem, (cudaStream_t)stream>>>(tb, a);
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
