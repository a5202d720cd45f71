// Tensor-core (tcgen05) 3x3x3 periodic convolution for the inner layers of the
// learned-guess network: implicit GEMM with BF16 operands from shared memory
// and the FP32 accumulator in tensor memory.
//
// One CTA computes a tile of 128 output voxels (16 rows y x 8 columns x of
// one z plane) for all C_out channels:
//   D[m][co] = sum_{tap, ci} A_tap[m][ci] W_tap[co][ci]
// with A_tap[m][ci] = in[ci][voxel m shifted by tap] (periodic).  The CTA
// stages the input brick the tile's 27 taps touch (3 planes x 18 rows x 10
// columns, "halo") once, in BF16, as planes of 8-channel chunks:
//   halo[chunk][hz][hy][hx][8 channels]     (16 bytes per voxel and chunk)
// In that layout the A operand of every tap is a plain shared-memory
// descriptor view of the halo (no per-tap copies): the tensor core's
// K-major no-swizzle operand is built of 8-row x 16-byte core matrices, and
// 8 consecutive output voxels along x are 8 consecutive 16-byte rows of one
// chunk plane; the next 8 (the next y row) start 10 voxels (160 bytes) on
// (stride-dimension offset), the next 8 input channels one chunk plane on
// (leading-dimension offset).  A tap is a start-address offset.  Weights
// are packed per tap the same way ([tap][chunk][co][8]; next 8 output
// channels 128 bytes on, next chunk C_out * 16 bytes on).
//
// One thread issues the MMAs (M = 128, N = C_out, K = 16 per instruction,
// 27 C_in / 16 of them); their completion is signalled on an mbarrier by
// tcgen05.commit; the four warps then read the accumulator rows of their
// TMEM lane quarter (tcgen05.ld 32x32b), add the bias, apply SiLU if asked,
// add a skip tensor if given and store FP32 [C][D][H][W].  The input may be
// read as the nearest-neighbour 2x upsampling of a half-size grid (the
// decoder's upsample fused into the load).  CTAs are persistent (as many as
// are resident; each loops over tiles), so weights that fit (27 taps <= 48
// KB) are loaded once per CTA; larger layers stream them per tile in three
// slabs of 9 taps (a slab buffer is reloaded after the MMAs reading it have
// completed).  Waits are bounded: on a timeout the kernel records an error
// code, waits (bounded) once more, releases its tensor memory and returns.
#include <cuda_bf16.h>
#include <stdint.h>

#include <type_traits>

#include "plan.h"

namespace {

constexpr int kTcThreads = 128;
constexpr int kHalo = 3 * 18 * 10;          // voxels of the staged input brick
constexpr int kChunkBytes = kHalo * 16;     // one 8-channel chunk plane
constexpr unsigned kSpinLimit = 1u << 20;   // mbarrier polls before giving up

template <int CIN, int COUT> struct TcCfg {
  static constexpr int NCH = CIN / 8;
  static constexpr int HALO_BYTES = NCH * kChunkBytes;
  static constexpr int TAP_BYTES = CIN * COUT * 2;                 // one tap of packed weights
  static constexpr int SLABS = 27 * TAP_BYTES > 64 * 1024 ? 3 : 1;
  static constexpr int TPS = 27 / SLABS;                           // taps per slab
  static constexpr int SLAB_BYTES = TPS * TAP_BYTES;
  static constexpr int SMEM = HALO_BYTES + SLAB_BYTES;
  static constexpr int TCOLS = COUT <= 32 ? 32 : (COUT <= 64 ? 64 : 128);   // TMEM columns (power of 2)
  // kind::f16 instruction descriptor: D FP32, A and B BF16, both K-major,
  // N = C_out, M = 128
  static constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(COUT >> 3) << 17) |
                                    ((uint32_t)(128 >> 4) << 24);
  static_assert(CIN % 16 == 0 && COUT % 16 == 0 && COUT <= 256, "tensor-core layer shape");
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor, no swizzle (version 1)
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (unsigned i = 0; i < kSpinLimit; ++i)
    if (mbar_try(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

template <int CIN, int COUT>
__global__ void __launch_bounds__(kTcThreads) k_conv3d_tc(const float* __restrict__ in,
                                                          const __nv_bfloat16* __restrict__ wpk,
                                                          const float* __restrict__ bias, float* __restrict__ out,
                                                          int D, int H, int W, int act,
                                                          const float* __restrict__ skip, int up, int nstore,
                                                          int* err) {
  using C = TcCfg<CIN, COUT>;
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* halo = smem;
  unsigned char* wsm = smem + C::HALO_BYTES;
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  __shared__ int failed;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ntx = W / 8, nty = H / 16;
  const int ntiles = ntx * nty * D;
  const int64_t HW = (int64_t)H * W, DHW = (int64_t)D * HW;
  // input grid: the output grid, or (up) half of it in every direction,
  // read as its nearest-neighbour 2x upsampling
  const int Di = up ? D / 2 : D, Hi = up ? H / 2 : H, Wi = up ? W / 2 : W;
  const int64_t HWi = (int64_t)Hi * Wi, DHWi = (int64_t)Di * HWi;
  const uint32_t bar_a = smem_u32(&bar);
  const uint32_t halo_a = smem_u32(halo), w_a = smem_u32(wsm);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tslot)),
                 "r"((uint32_t)C::TCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_a) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    failed = 0;
  }
  auto load_slab = [&](int s) {
    const uint4* src = reinterpret_cast<const uint4*>(wpk) + (int64_t)s * (C::SLAB_BYTES / 16);
    for (int i = tid; i < C::SLAB_BYTES / 16; i += kTcThreads) reinterpret_cast<uint4*>(wsm)[i] = __ldg(src + i);
  };
  // one-slab layers keep their weights for every tile of the CTA
  if (C::SLABS == 1) load_slab(0);
  uint32_t ncommit = 0;     // commits so far: the next wait is on parity (ncommit - 1) & 1
  // persistent over tiles (tile = 16 rows x 8 columns of one z plane)
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    int b = tile;
    const int x0 = (b % ntx) * 8;
    b /= ntx;
    const int y0 = (b % nty) * 16;
    const int z = b / nty;
    // input brick in BF16: one 16-byte chunk (8 channels of one voxel) per item
    for (int e = tid; e < C::NCH * kHalo; e += kTcThreads) {
      const int v = e % kHalo, ch = e / kHalo;
      const int hx = v % 10, hy = (v / 10) % 18, hz = v / 180;
      int gz = wrap(z + hz - 1, D), gy = wrap(y0 + hy - 1, H), gx = wrap(x0 + hx - 1, W);
      if (up) { gz >>= 1; gy >>= 1; gx >>= 1; }
      const float* p = in + (int64_t)(ch * 8) * DHWi + gz * HWi + (int64_t)gy * Wi + gx;
      uint32_t u[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const __nv_bfloat162 h2 = __floats2bfloat162_rn(__ldg(p + (2 * q) * DHWi), __ldg(p + (2 * q + 1) * DHWi));
        u[q] = *reinterpret_cast<const uint32_t*>(&h2);
      }
      *reinterpret_cast<uint4*>(halo + ch * kChunkBytes + v * 16) = make_uint4(u[0], u[1], u[2], u[3]);
    }
    for (int s = 0; s < C::SLABS; ++s) {
      if (s > 0) {
        // the previous slab's MMAs must be done before its buffer is reused
        if (!mbar_wait(bar_a, (ncommit - 1) & 1u) && tid == 0) { failed = 1; atomicExch(err, 1); }
        __syncthreads();
        if (failed) break;
      }
      if (C::SLABS > 1) load_slab(s);
      // make the generic-proxy shared-memory writes visible to the tensor core
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (tid == 0) {
        const uint32_t tbase = tslot;
        for (int tl = 0; tl < C::TPS; ++tl) {
          const int t = s * C::TPS + tl;
          const int dz = t / 9, dy = (t / 3) % 3, dx = t % 3;
          const uint32_t a0 = halo_a + (uint32_t)(((dz * 18 + dy) * 10 + dx) * 16);
          const uint32_t b0 = w_a + (uint32_t)(tl * C::TAP_BYTES);
#pragma unroll
          for (int kk = 0; kk < CIN / 16; ++kk) {
            const uint64_t ad = sdesc(a0 + (uint32_t)(2 * kk * kChunkBytes), kChunkBytes, 160);
            const uint64_t bd = sdesc(b0 + (uint32_t)(2 * kk * COUT * 16), COUT * 16, 128);
            mma_bf16(tbase, ad, bd, C::IDESC, (t > 0 || kk > 0) ? 1u : 0u);
          }
        }
        mma_commit(bar_a);
      }
      ++ncommit;
    }
    if (failed) break;
    // completion of the tile's last commit (bounded; every thread waits, the
    // decision to go on is taken together)
    if (!mbar_wait(bar_a, (ncommit - 1) & 1u)) failed = 2;
    __syncthreads();
    if (failed) {
      if (tid == 0) atomicExch(err, 2);
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // accumulator row m = warp * 32 + lane -> voxel (z, y0 + m / 8, x0 + m % 8)
    const int m = warp * 32 + lane;
    const int y = y0 + (m >> 3), x = x0 + (m & 7);
    const int64_t off = z * HW + (int64_t)y * W + x;
    float* o = out + off;
    const float* sk = skip ? skip + off : nullptr;
    const uint32_t tbase = tslot;
#pragma unroll
    for (int cb = 0; cb < COUT / 16; ++cb) {
      float v[16];
      tmem_ld16(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cb * 16), v);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int co = cb * 16 + i;
        if (co >= nstore) continue;
        float r = v[i] + (bias ? __ldg(bias + co) : 0.0f);
        if (act) r = r / (1.0f + __expf(-r));
        if (sk) r += __ldg(sk + (int64_t)co * DHW);
        o[(int64_t)co * DHW] = r;
      }
    }
    // the accumulator and the halo are reused by the next tile
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
  }
  // a timed-out wait: one more bounded wait for the MMAs in flight before
  // the tensor memory is released
  __syncthreads();
  if (failed && ncommit > 0) mbar_wait(bar_a, (ncommit - 1) & 1u);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tslot), "r"((uint32_t)C::TCOLS)
                 : "memory");
}

// z-pipelined form for layers whose weights stay in shared memory: a CTA
// owns one column of tiles (16 rows x 8 columns) and walks zc planes of it.
// The input brick is a ring of 4 planes (plane p in slot p mod 4; the taps
// of output plane z read slots of planes z-1, z, z+1), so each step loads
// one new plane, and it loads it while the MMAs of the current plane run;
// the accumulator is double-buffered in TMEM, so the MMAs of plane z+1 run
// while the epilogue of plane z drains.
template <int CIN, int COUT> struct TczCfg {
  static constexpr int NCH = CIN / 8;
  static constexpr int PLANE = 18 * 10 * 16;            // one brick plane of one chunk (bytes)
  static constexpr int CHUNK = 4 * PLANE;                // a chunk's ring of 4 planes
  static constexpr int RING_BYTES = NCH * CHUNK;
  static constexpr int SMEM = RING_BYTES + TcCfg<CIN, COUT>::SLAB_BYTES;
  static constexpr int TCOLS = 2 * COUT <= 32 ? 32 : (2 * COUT <= 64 ? 64 : (2 * COUT <= 128 ? 128 : 256));
};

template <int CIN, int COUT>
__global__ void __launch_bounds__(kTcThreads) k_conv3d_tcz(const float* __restrict__ in,
                                                           const __nv_bfloat16* __restrict__ wpk,
                                                           const float* __restrict__ bias, float* __restrict__ out,
                                                           int D, int H, int W, int act,
                                                           const float* __restrict__ skip, int up, int nstore,
                                                           int zc, int* err) {
  using C = TcCfg<CIN, COUT>;
  using Z = TczCfg<CIN, COUT>;
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* ring = smem;
  unsigned char* wsm = smem + Z::RING_BYTES;
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  __shared__ int failed;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ntx = W / 8, ncol = ntx * (H / 16);
  const int col = blockIdx.x % ncol, chunk = blockIdx.x / ncol;
  const int x0 = (col % ntx) * 8, y0 = (col / ntx) * 16;
  const int z0 = chunk * zc, z1 = min(D, z0 + zc);
  const int64_t HW = (int64_t)H * W, DHW = (int64_t)D * HW;
  const int Di = up ? D / 2 : D, Hi = up ? H / 2 : H, Wi = up ? W / 2 : W;
  const int64_t HWi = (int64_t)Hi * Wi, DHWi = (int64_t)Di * HWi;
  const uint32_t bar_a = smem_u32(&bar);
  const uint32_t ring_a = smem_u32(ring), w_a = smem_u32(wsm);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tslot)),
                 "r"((uint32_t)Z::TCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_a) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    failed = 0;
  }
  {
    const uint4* src = reinterpret_cast<const uint4*>(wpk);
    for (int i = tid; i < C::SLAB_BYTES / 16; i += kTcThreads) reinterpret_cast<uint4*>(wsm)[i] = __ldg(src + i);
  }
  // input plane p (periodic) into ring slot p & 3: items (chunk, voxel), the
  // loads of up to 4 items issued before their stores
  auto load_plane = [&](int p) {
    const int gz0 = wrap(p, D);
    const int gz = up ? gz0 >> 1 : gz0;
    unsigned char* dst = ring + (p & 3) * Z::PLANE;
    constexpr int NIT = Z::NCH * 180;
    for (int e0 = 0; e0 < NIT; e0 += 4 * kTcThreads) {
      float f[4][8];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int e = e0 + u * kTcThreads + tid;
        if (e < NIT) {
          const int v = e % 180, ch = e / 180;
          int gy = wrap(y0 + v / 10 - 1, H), gx = wrap(x0 + v % 10 - 1, W);
          if (up) { gy >>= 1; gx >>= 1; }
          const float* q = in + (int64_t)(ch * 8) * DHWi + gz * HWi + (int64_t)gy * Wi + gx;
#pragma unroll
          for (int c = 0; c < 8; ++c) f[u][c] = __ldg(q + c * DHWi);
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int e = e0 + u * kTcThreads + tid;
        if (e < NIT) {
          const int v = e % 180, ch = e / 180;
          uint32_t w4[4];
#pragma unroll
          for (int q2 = 0; q2 < 4; ++q2) {
            const __nv_bfloat162 h2 = __floats2bfloat162_rn(f[u][2 * q2], f[u][2 * q2 + 1]);
            w4[q2] = *reinterpret_cast<const uint32_t*>(&h2);
          }
          *reinterpret_cast<uint4*>(dst + ch * Z::CHUNK + v * 16) = make_uint4(w4[0], w4[1], w4[2], w4[3]);
        }
      }
    }
  };
  auto publish = [&]() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  };
  // MMAs of output plane z into accumulator buffer z & 1 (one thread)
  auto issue = [&](int z) {
    const uint32_t acc = tslot + (uint32_t)((z & 1) * COUT);
    for (int t = 0; t < 27; ++t) {
      const int dz = t / 9, dy = (t / 3) % 3, dx = t % 3;
      const uint32_t a0 = ring_a + (uint32_t)(((z - 1 + dz) & 3) * Z::PLANE + (dy * 10 + dx) * 16);
      const uint32_t b0 = w_a + (uint32_t)(t * C::TAP_BYTES);
#pragma unroll
      for (int kk = 0; kk < CIN / 16; ++kk) {
        const uint64_t ad = sdesc(a0 + (uint32_t)(2 * kk * Z::CHUNK), Z::CHUNK, 160);
        const uint64_t bd = sdesc(b0 + (uint32_t)(2 * kk * COUT * 16), COUT * 16, 128);
        mma_bf16(acc, ad, bd, C::IDESC, (t > 0 || kk > 0) ? 1u : 0u);
      }
    }
    mma_commit(bar_a);
  };
  // prologue: planes z0-1, z0, z0+1, the MMAs of z0
  load_plane(z0 - 1);
  load_plane(z0);
  load_plane(z0 + 1);
  publish();
  if (tid == 0) issue(z0);
  uint32_t ncommit = 1;
  const int m = warp * 32 + lane;
  const int y = y0 + (m >> 3), x = x0 + (m & 7);
  for (int z = z0; z < z1; ++z) {
    if (z + 1 < z1) load_plane(z + 2);     // overlaps the MMAs of z
    const int64_t off = z * HW + (int64_t)y * W + x;
    // the skip values of this thread's voxel, loaded before the wait
    float skv[COUT];
#pragma unroll
    for (int co = 0; co < COUT; ++co) skv[co] = (skip && co < nstore) ? __ldg(skip + off + (int64_t)co * DHW) : 0.0f;
    publish();
    if (!mbar_wait(bar_a, (ncommit - 1) & 1u)) failed = 1;
    __syncthreads();
    if (failed) break;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (z + 1 < z1) {
      if (tid == 0) issue(z + 1);         // overlaps the epilogue of z
      ++ncommit;
    }
    float* o = out + off;
    const uint32_t acc = tslot + (uint32_t)((z & 1) * COUT) + ((uint32_t)(warp * 32) << 16);
#pragma unroll
    for (int cb = 0; cb < COUT / 16; ++cb) {
      float v[16];
      tmem_ld16(acc + (uint32_t)(cb * 16), v);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int co = cb * 16 + i;
        if (co >= nstore) continue;
        float r = v[i] + (bias ? __ldg(bias + co) : 0.0f);
        if (act) r = r / (1.0f + __expf(-r));
        o[(int64_t)co * DHW] = r + skv[co];
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  __syncthreads();
  if (failed) {
    if (tid == 0) atomicExch(err, 3);
    mbar_wait(bar_a, (ncommit - 1) & 1u);    // bounded, before the tensor memory is released
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tslot), "r"((uint32_t)Z::TCOLS)
                 : "memory");
}

// [co][ci][27] -> [tap][ci / 8][co][ci % 8]
__global__ void k_pack_tc(const __nv_bfloat16* __restrict__ w, __nv_bfloat16* __restrict__ out, int cin, int cout) {
  const int n = 27 * cin * cout;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int q = i % 8, co = (i / 8) % cout, ch = (i / (8 * cout)) % (cin / 8), t = i / (cout * cin);
    const int ci = ch * 8 + q;
    out[i] = w[((int64_t)co * cin + ci) * 27 + t];
  }
}

// the dynamic shared-memory attribute of a kernel, set once per device (the
// plans' registry of granted sizes, shared with the other passes)
template <typename K>
int tc_smem(K kern, int bytes) {
  int dev = 0;
  GB_CUDA(cudaGetDevice(&dev));
  const void* key = reinterpret_cast<const void*>(kern);
  if (gb_smem_granted(key, dev) >= bytes) return 0;
  GB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  gb_smem_grant(key, dev, bytes);
  return 0;
}

template <int CIN, int COUT>
int launch_tc(const float* in, const __nv_bfloat16* wpk, const float* bias, float* out, int D, int H, int W, int act,
              const float* skip, int up, int nstore, int* err, cudaStream_t st) {
  using C = TcCfg<CIN, COUT>;
  int rc = 0;
  if constexpr (C::SLABS == 1) {
    // z-pipelined kernel: a CTA walks a column of tiles along z
    using Z = TczCfg<CIN, COUT>;
    if ((rc = tc_smem(k_conv3d_tcz<CIN, COUT>, Z::SMEM))) return rc;
    int dev = 0, nsm = 0;
    GB_CUDA(cudaGetDevice(&dev));
    GB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    // about 8 CTAs per SM: z chunks of the columns (a chunk of zc planes
    // loads zc + 2 input planes)
    const int ncol = (W / 8) * (H / 16);
    const int target = 8 * (nsm > 0 ? nsm : 152);
    int nchunk = (target + ncol - 1) / ncol;
    if (nchunk < 1) nchunk = 1;
    if (nchunk > D) nchunk = D;
    const int zc = (D + nchunk - 1) / nchunk;
    nchunk = (D + zc - 1) / zc;
    k_conv3d_tcz<CIN, COUT><<<ncol * nchunk, kTcThreads, Z::SMEM, st>>>(in, wpk, bias, out, D, H, W, act, skip, up,
                                                                      nstore, zc, err);
  } else {
    if ((rc = tc_smem(k_conv3d_tc<CIN, COUT>, C::SMEM))) return rc;
    const int ntiles = (W / 8) * (H / 16) * D;
    k_conv3d_tc<CIN, COUT><<<ntiles, kTcThreads, C::SMEM, st>>>(in, wpk, bias, out, D, H, W, act, skip, up, nstore,
                                                                 err);
  }
  GB_CHECK_LAUNCH();
  gb_count_launch();
  return 0;
}

template <typename F>
bool tc_dispatch(int cin, int cout, F&& f) {
#define GB_TC_CASE(A, B)                                                      \
  if (cin == A && cout == B) {                                                \
    f(std::integral_constant<int, A>{}, std::integral_constant<int, B>{});    \
    return true;                                                              \
  }
  GB_TC_CASE(16, 16) GB_TC_CASE(16, 32) GB_TC_CASE(32, 16) GB_TC_CASE(32, 32) GB_TC_CASE(32, 48)
  GB_TC_CASE(48, 32) GB_TC_CASE(48, 48) GB_TC_CASE(48, 64) GB_TC_CASE(64, 48) GB_TC_CASE(64, 64)
#undef GB_TC_CASE
  return false;
}

}  // namespace

extern "C" {

int gbofdft_nn_conv3d_tc_supported(int cin, int cout, int D, int H, int W) {
  if (D < 1 || H % 16 || W % 8) return 0;
  return tc_dispatch(cin, cout, [](auto, auto) {}) ? 1 : 0;
}

int gbofdft_nn_conv3d_tc_pack(const void* w, int cin, int cout, void* out, void* stream) {
  GB_REQUIRE(w && out, "nn_conv3d_tc_pack: null argument");
  GB_REQUIRE(cin % 8 == 0 && cout > 0, "nn_conv3d_tc_pack: c_in must be a multiple of 8");
  const int n = 27 * cin * cout;
  k_pack_tc<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const __nv_bfloat16*>(w),
                                                                reinterpret_cast<__nv_bfloat16*>(out), cin, cout);
  GB_CHECK_LAUNCH();
  gb_count_launch();
  return 0;
}

int gbofdft_nn_conv3d_tc(const void* in, int cin, const void* wpk, const void* bias, void* out, int cout, int nstore,
                         int D, int H, int W, int act, const void* skip, int up, int* err, void* stream) {
  GB_REQUIRE(in && wpk && out && err, "nn_conv3d_tc: null argument");
  GB_REQUIRE(nstore >= 1 && nstore <= cout, "nn_conv3d_tc: nstore %d outside [1, %d]", nstore, cout);
  GB_REQUIRE(gbofdft_nn_conv3d_tc_supported(cin, cout, D, H, W),
             "nn_conv3d_tc: no tensor-core kernel for %d -> %d channels on %d x %d x %d", cin, cout, D, H, W);
  GB_REQUIRE(!up || (D % 2 == 0 && H % 2 == 0 && W % 2 == 0), "nn_conv3d_tc: upsampled input needs even extents");
  int rc = 0;
  tc_dispatch(cin, cout, [&](auto a, auto b) {
    rc = launch_tc<decltype(a)::value, decltype(b)::value>(
        reinterpret_cast<const float*>(in), reinterpret_cast<const __nv_bfloat16*>(wpk),
        reinterpret_cast<const float*>(bias), reinterpret_cast<float*>(out), D, H, W, act,
        reinterpret_cast<const float*>(skip), up, nstore, err, (cudaStream_t)stream);
  });
  return rc;
}

}  // extern "C"
