// The warm-start network's 3 x 3 convolutions on the 5th-generation tensor
// cores: an implicit GEMM with TMA-staged operands, tcgen05.mma accumulating
// in tensor memory, and the bias / ReLU / skip epilogue fused.  No reference
// counterpart (the reference starts ERA from ones, ptychography/era.py:480-486;
// this network computes the learned warm start that replaces that start).
//
//   out[p][co] = act(sum_{tap, ci} X[p + tap offset][ci] Wt[co][tap C_in + ci] + bias[co]) (+ skip[p][co])
//
// with X, out, skip NHWC bf16 and Wt[C_out][9 C_in] bf16 (k = (ky*3 + kx) C_in
// + ci, the layout of the im2col path), FP32 accumulation.
//
// A tile is 128 consecutive output pixels (one image row of 128, or 128 / W
// whole rows of a narrower image): the MMA's M = 128, N = C_out (32..256, a
// multiple of 32 up to 128), K = 9 C_in walked as (tap, 64-channel chunk) stages of
// four K = 16 steps.  For each stage one TMA load brings the 128 input pixels
// shifted by the tap ((ky - 1, kx - 1): the tensor map's out-of-bounds zero
// fill is the convolution's zero padding) and one brings the weights' matching
// C_out x 64 slice, both in the 128-byte-swizzled K-major layout the MMA
// reads (64-byte swizzle when C_in = 32).  No im2col buffer is written.
// A layer whose tiles are single image rows of 64 input channels (C_out up
// to 64) stages instead the tile's three input rows with a one-pixel halo
// and keeps the nine weight taps resident: the kx shift of a tap is a start
// one or two swizzled rows into the staged row (halo staging, see the kernel).
//
// Roles (persistent CTAs of 192 threads, one or two per SM by the size of the
// layer's stage ring):
//   warp 4, one lane: TMA producer over a ring of 4-8 stages;
//   warp 5, one lane: MMA issuer; accumulators double-buffered in TMEM so the
//     epilogue of one tile overlaps the MMAs of the next;
//   warps 0-3: epilogue, warp w reading TMEM lanes 32w..32w+31 (its 32 pixels).
// Every mbarrier wait is bounded: past the limit the kernel records an error
// flag, stops issuing, waits (bounded) for its copies and MMAs in flight, frees
// its tensor memory and returns; the host reads the flag.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <mutex>

#include "../../include/ptycho_gb300.h"
#include "engine.h"

namespace pty {
namespace {

constexpr int kTileM = 128;
constexpr int kChunk = 64;            // input channels per stage
constexpr int kStages = 4;            // ring depth of a layer running one CTA per SM
constexpr int kMaxStages = 8;
#ifndef PTY_WS_RING_MAX
#define PTY_WS_RING_MAX kMaxStages   // deepest ring ring_depth() picks (a tuning bound, 4..8)
#endif
constexpr int kThreads = 192;
constexpr int kMaxCout = 128;
constexpr int kAccCols = 256;         // TMEM columns: two accumulators of up to 128
// at least this much dynamic shared memory per CTA, so that at most two CTAs
// share an SM and their tensor-memory allocations (kAccCols each, 512 columns
// per SM) never wait for another CTA's; a layer whose stage ring fits in
// kTwoPerSm bytes runs two CTAs per SM (twice the TMA bytes in flight)
constexpr size_t kMinSmem = 77 * 1024;
constexpr size_t kTwoPerSm = 112 * 1024;
constexpr size_t kHaloSmem = 227 * 1024;   // the halo-staging ring fills one SM's shared memory
constexpr unsigned kSpinLimit = 1u << 26;

struct ConvParams {
  int B, H, W, Cin, Cout;
  int wbox, rows;          // input box: wbox pixels x rows image rows (wbox * rows = 128)
  int xtiles;              // tiles per image row (W / 128 when W >= 128, else 1)
  int tiles;               // B * (H / rows) * xtiles
  int chunks;              // ceil(Cin / 64)
  int chunk_ch;            // channels per chunk (64, or Cin when Cin < 64)
  int stages;              // TMA ring depth (<= kMaxStages)
  int halo;                // one image row per tile, C_in = 64: halo-row staging (see the kernel)
  int relu;
  const float* bias;       // [Cout]
  const __nv_bfloat16* skip;   // [P][Cout] or nullptr
  __nv_bfloat16* out;          // [P][Cout]
  __nv_bfloat16* act;          // [P][Cout] the activation before the skip, or nullptr
  float* out32;                // [P][Cout] raw FP32 sums instead of out (no bias, activation, skip)
  int* err;                    // device error flag (set on a wait timeout)
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase with the given parity: false (and the CTA's abort
// flag and the global error flag set) after kSpinLimit polls, or at once when
// another role has already aborted.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, volatile int* abort,
                                          int* err) {
  for (unsigned i = 0; i < kSpinLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort) return false;
  }
  *abort = 1;
  atomicExch(err, 1);
  return false;
}
// The same for a whole warp, which leaves together (success or timeout), as
// the warp-collective tensor-memory loads after it require.
__device__ __forceinline__ bool mbar_wait_warp(uint64_t* bar, unsigned parity, volatile int* abort,
                                               int* err) {
  for (unsigned i = 0; i < kSpinLimit; ++i) {
    const bool done = mbar_try_wait(bar, parity);
    if (__all_sync(0xffffffffu, done)) return true;
    if (__any_sync(0xffffffffu, *abort != 0)) return false;
  }
  if ((threadIdx.x & 31) == 0) {
    *abort = 1;
    atomicExch(err, 1);
  }
  return false;
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0,
                                            int c1, int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%3, %4, %5, %6}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
      : "memory");
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0,
                                            int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1)
      : "memory");
}

// Shared-memory matrix descriptor (tcgen05): start address >> 4 in bits 0-13,
// leading-dimension byte offset >> 4 in 16-29 (unused by swizzled K-major
// layouts; 1), stride byte offset >> 4 in 32-45 (8 rows of the swizzle atom),
// the descriptor version 1 in bits 46-47, the swizzle mode in bits 61-63
// (2: 128-byte swizzle, 4: 64-byte swizzle).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, int swz_bytes) {
  const uint64_t sbo = (uint64_t)(8 * swz_bytes) >> 4;
  const uint64_t mode = swz_bytes == 128 ? 2ull : 4ull;
  return (uint64_t)((addr >> 4) & 0x3FFF) | (1ull << 16) | (sbo << 32) | (1ull << 46) | (mode << 61);
}
// The same for a 128-byte-swizzled K-major matrix whose first row is not at
// the start of a 1024-byte swizzle pattern.  The MMA forms the swizzle from
// the absolute shared-memory address (as the TMA that wrote the rows did):
// a start one or two rows in needs no base offset, just as the K steps'
// starts 32-96 bytes into a row need none.
__device__ __forceinline__ uint64_t smem_desc_row(uint32_t addr) { return smem_desc(addr, 128); }

// Instruction descriptor, kind::f16: D f32 (bits 4-5 = 1), A and B bf16 (bits
// 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in bits 17-22,
// M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t da, uint64_t db, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// 32 consecutive accumulator columns of this warp's 32 TMEM lanes
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
        "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

constexpr int kHaloPix = kTileM + 2;   // a halo row: the tile's 128 pixels and one on each side

struct __align__(8) SmemCtl {
  uint64_t wfull;                      // halo staging: the resident weights have landed
  uint64_t full[kMaxStages];
  uint64_t empty[kMaxStages];
  uint64_t acc_full[2];
  uint64_t acc_empty[2];
  uint64_t drain;
  uint32_t tmem_base;
  int abort;
  float bias[kMaxCout];
};

// tile t -> (image b, first row y0, first column x0)
__device__ __forceinline__ void tile_origin(const ConvParams& p, int t, int& b, int& y0, int& x0) {
  const int xt = t % p.xtiles;
  const int rt = t / p.xtiles;
  const int rows_per_img = p.H / p.rows;
  b = rt / rows_per_img;
  y0 = (rt % rows_per_img) * p.rows;
  x0 = xt * p.wbox;
}

__global__ void __launch_bounds__(kThreads, 1)
    ws_conv_tc_kernel(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmW,
                      const __grid_constant__ CUtensorMap tmH, const ConvParams p) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // stage buffers at a 1024-byte boundary (the 128-byte swizzle's atom)
  const uint32_t raw = smem_u32(smem_raw);
  unsigned char* base = smem_raw + ((1024 - (raw & 1023)) & 1023);
  const int nst = p.stages;
  const int a_bytes = kTileM * p.chunk_ch * 2;            // 16 KB (8 KB when C_in = 32)
  const int b_bytes = p.Cout * p.chunk_ch * 2;
  // Halo staging (a tile of one image row, C_in = 64): the nine taps' weights
  // stay resident (wtap bytes each), and a stage holds the three input rows
  // y0 - 1 .. y0 + 1 of the tile, 130 pixels each (hrow bytes); tap (ky, kx)
  // reads row ky from pixel kx on, a start one or two 128-byte rows into the
  // swizzle pattern (smem_desc_row).  Three 17 KB loads per tile instead of
  // nine 16 KB loads plus the weights.
  const int wtap = ((p.Cout * 128 + 1023) / 1024) * 1024;
  const int hrow = ((kHaloPix * 128 + 1023) / 1024) * 1024;
  unsigned char* wres = base;
  unsigned char* ring = p.halo ? base + 9 * wtap : base;
  const int stage_bytes = p.halo ? 3 * hrow : ((a_bytes + b_bytes + 1023) / 1024) * 1024;
  SmemCtl* ctl = reinterpret_cast<SmemCtl*>(ring + nst * stage_bytes);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int swz = p.chunk_ch * 2;                         // 128 or 64 bytes per row

  for (int i = threadIdx.x; i < p.Cout; i += kThreads) ctl->bias[i] = p.bias ? p.bias[i] : 0.f;
  if (threadIdx.x == 0) {
    for (int s = 0; s < nst; ++s) {
      mbar_init(&ctl->full[s], 1);
      mbar_init(&ctl->empty[s], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&ctl->acc_full[i], 1);
      mbar_init(&ctl->acc_empty[i], 4);
    }
    mbar_init(&ctl->drain, 1);
    mbar_init(&ctl->wfull, 1);
    ctl->abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&ctl->tmem_base)),
                 "r"(kAccCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = ctl->tmem_base;
  volatile int* abort = &ctl->abort;
  const int ksteps = p.chunk_ch / 16;
  const int nstage_per_tile = p.halo ? 1 : 9 * p.chunks;
  const uint32_t idesc = instr_desc(kTileM, p.Cout);
  const uint32_t acc_stride = 128u;                        // column offset of the second accumulator

  if (warp == 4) {
    // ------------------------------------------------ TMA producer
    if (lane == 0) {
      int q = 0, rs = 0, rph = 0;   // ring position: q = stages used, rs = q mod nst, rph = its phase
      bool ok = true;
      if (p.halo) {
        // the nine taps' weights, once per CTA
        mbar_expect_tx(&ctl->wfull, (unsigned)(9 * p.Cout * 128));
        for (int tap = 0; tap < 9; ++tap) tma_load_2d(wres + tap * wtap, &tmW, &ctl->wfull, tap * p.Cin, 0);
      }
      for (int t = blockIdx.x; t < p.tiles && ok; t += gridDim.x) {
        int b, y0, x0;
        tile_origin(p, t, b, y0, x0);
        for (int st = 0; st < nstage_per_tile && ok; ++st, ++q, rs = (rs + 1 == nst) ? 0 : rs + 1, rph ^= (rs == 0)) {
          const int s = rs, ph = rph;
          if (!mbar_wait(&ctl->empty[s], ph ^ 1, abort, p.err)) { ok = false; break; }
          unsigned char* sa = ring + s * stage_bytes;
          if (p.halo) {
            mbar_expect_tx(&ctl->full[s], (unsigned)(3 * kHaloPix * 128));
            for (int ky = 0; ky < 3; ++ky)
              tma_load_4d(sa + ky * hrow, &tmH, &ctl->full[s], 0, x0 - 1, y0 + ky - 1, b);
            continue;
          }
          const int tap = st / p.chunks, ch = st % p.chunks;
          const int ky = tap / 3, kx = tap % 3;
          unsigned char* sb = sa + a_bytes;
          mbar_expect_tx(&ctl->full[s], (unsigned)(a_bytes + b_bytes));
          tma_load_4d(sa, &tmX, &ctl->full[s], ch * p.chunk_ch, x0 + kx - 1, y0 + ky - 1, b);
          tma_load_2d(sb, &tmW, &ctl->full[s], tap * p.Cin + ch * p.chunk_ch, 0);
        }
      }
      // copies issued but never consumed (after an abort) finish before exit
      if (!ok) {
        for (int k = 0; k < nst; ++k) {
          const int qq = q - 1 - k;
          if (qq < 0) break;
          const int s = qq % nst, ph = (qq / nst) & 1;
          for (unsigned i = 0; i < kSpinLimit && !mbar_try_wait(&ctl->full[s], ph); ++i) {
          }
        }
        if (p.halo)
          for (unsigned i = 0; i < kSpinLimit && !mbar_try_wait(&ctl->wfull, 0); ++i) {
          }
      }
    }
  } else if (warp == 5) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      int q = 0, rs = 0, rph = 0, local = 0;
      bool ok = true;
      if (p.halo && !mbar_wait(&ctl->wfull, 0, abort, p.err)) ok = false;
      if (p.halo) asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int t = blockIdx.x; t < p.tiles && ok; t += gridDim.x, ++local) {
        const int buf = local & 1, use = local >> 1;
        if (!mbar_wait(&ctl->acc_empty[buf], (use & 1) ^ 1, abort, p.err)) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t d = tmem + buf * acc_stride;
        for (int st = 0; st < nstage_per_tile; ++st, ++q, rs = (rs + 1 == nst) ? 0 : rs + 1, rph ^= (rs == 0)) {
          const int s = rs, ph = rph;
          if (!mbar_wait(&ctl->full[s], ph, abort, p.err)) { ok = false; break; }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t sa = smem_u32(ring + s * stage_bytes);
          if (p.halo) {
            const uint32_t wb = smem_u32(wres);
            for (int tap = 0; tap < 9; ++tap) {
              const int ky = tap / 3, kx = tap % 3;
              const uint32_t a0 = sa + ky * hrow + kx * 128, b0 = wb + tap * wtap;
              for (int k = 0; k < 4; ++k)
                mma_bf16(d, smem_desc_row(a0 + 32 * k), smem_desc(b0 + 32 * k, 128), idesc,
                         (tap > 0 || k > 0) ? 1u : 0u);
            }
            mma_commit(&ctl->empty[s]);
            continue;
          }
          const uint32_t sb = sa + a_bytes;
          for (int k = 0; k < ksteps; ++k) {
            // K = 16 bf16 = 32 bytes along the swizzled row
            mma_bf16(d, smem_desc(sa + 32 * k, swz), smem_desc(sb + 32 * k, swz), idesc,
                     (st > 0 || k > 0) ? 1u : 0u);
          }
          mma_commit(&ctl->empty[s]);   // stage free once these MMAs have read it
        }
        if (!ok) break;
        mma_commit(&ctl->acc_full[buf]);
      }
      // every MMA issued has completed before the tensor memory is freed
      mma_commit(&ctl->drain);
      for (unsigned i = 0; i < kSpinLimit && !mbar_try_wait(&ctl->drain, 0); ++i) {
      }
    }
  } else {
    // ------------------------------------------------ epilogue (warps 0-3)
    int local = 0;
    for (int t = blockIdx.x; t < p.tiles; t += gridDim.x, ++local) {
      const int buf = local & 1, use = local >> 1;
      int b, y0, x0;
      tile_origin(p, t, b, y0, x0);
      const int r = warp * 32 + lane;                    // pixel row of the tile
      const int y = y0 + r / p.wbox, x = x0 + r % p.wbox;
      const size_t pix = ((size_t)b * p.H + y) * p.W + x;
      // the first 32 skip channels are loaded while the tile's MMAs run
      uint4 sk0[4];
      if (p.skip && !p.out32) {
#pragma unroll
        for (int q4 = 0; q4 < 4; ++q4) sk0[q4] = *reinterpret_cast<const uint4*>(p.skip + pix * p.Cout + 8 * q4);
      }
      if (!mbar_wait_warp(&ctl->acc_full[buf], use & 1, abort, p.err)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t tbase = tmem + buf * acc_stride + ((uint32_t)(warp * 32) << 16);
      for (int c0 = 0; c0 < p.Cout; c0 += 32) {
        float v[32];
        tmem_ld32(tbase + c0, v);
        if (c0 + 32 >= p.Cout) {
          // accumulator fully read: the MMA warp may reuse it
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0) mbar_arrive(&ctl->acc_empty[buf]);
        }
        if (p.out32) {
          float* o32 = p.out32 + pix * p.Cout + c0;
#pragma unroll
          for (int q4 = 0; q4 < 8; ++q4)
            *reinterpret_cast<float4*>(o32 + 4 * q4) = make_float4(v[4 * q4], v[4 * q4 + 1], v[4 * q4 + 2], v[4 * q4 + 3]);
          continue;
        }
        const __nv_bfloat16* sk = p.skip ? p.skip + pix * p.Cout + c0 : nullptr;
        __nv_bfloat16* o = p.out + pix * p.Cout + c0;
        __nv_bfloat16* ao = p.act ? p.act + pix * p.Cout + c0 : nullptr;
#pragma unroll
        for (int q4 = 0; q4 < 4; ++q4) {
          uint4 skv = make_uint4(0u, 0u, 0u, 0u);
          if (sk) skv = c0 == 0 ? sk0[q4] : *reinterpret_cast<const uint4*>(sk + 8 * q4);
          const __nv_bfloat162* s2 = reinterpret_cast<const __nv_bfloat162*>(&skv);
          uint4 ov, av;
          __nv_bfloat162* o2 = reinterpret_cast<__nv_bfloat162*>(&ov);
          __nv_bfloat162* a2 = reinterpret_cast<__nv_bfloat162*>(&av);
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            float a0 = v[8 * q4 + 2 * e] + ctl->bias[c0 + 8 * q4 + 2 * e];
            float a1 = v[8 * q4 + 2 * e + 1] + ctl->bias[c0 + 8 * q4 + 2 * e + 1];
            if (p.relu) {
              a0 = fmaxf(a0, 0.f);
              a1 = fmaxf(a1, 0.f);
            }
            __nv_bfloat162 h = __floats2bfloat162_rn(a0, a1);
            a2[e] = h;
            if (sk) {
              const float2 sf = __bfloat1622float2(s2[e]);
              const float2 hf = __bfloat1622float2(h);
              h = __floats2bfloat162_rn(hf.x + sf.x, hf.y + sf.y);
            }
            o2[e] = h;
          }
          *reinterpret_cast<uint4*>(o + 8 * q4) = ov;
          if (ao) *reinterpret_cast<uint4*>(ao + 8 * q4) = av;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kAccCols)
                 : "memory");
  }
}


// ---------------------------------------------------------------- weight gradient
//
//   dW[co][tap C_in + ci] = sum_p dZ[p][co] X[p shifted by tap][ci]
//
// as a GEMM with the pixels on K: D[k][co] with k = tap C_in + ci on the MMA's
// M (128 rows: 128 / C_in taps per M tile) and co on N.  Both operands are
// K-major, i.e. pixel-contiguous: XS[s][ci][p] = X[p shifted by s - 1 along
// x][ci] (three copies, so that the TMA's innermost coordinate, a pixel
// column, never carries the +-1 tap offset: it stays a multiple of the
// chunk) and dZT[co][p].  A stage is one chunk of 64 pixels of an image row
// (32 when W = 32): per tap of the M tile one box (chunk, 1 row, 1 image,
// C_in channels, 1 copy) at row y + ky - 1 of copy kx (rows outside the
// image read the zero fill), and one box (chunk, N) of dZT (rows past C_out
// read zeros, so C_out < 16 runs as N = 16).  Work items are (M tile, pixel
// range) pairs; each accumulates its range in tensor memory and writes an
// FP32 partial [split][k][co]; ws_wgrad_reduce_kernel sums the splits in
// order (deterministic).
struct WgradParams {
  int B, H, W, Cin, Cout, npad;  // npad: B-operand rows (C_out rounded up to 16)
  int kchunk;                    // pixels per stage
  int xtiles;                    // W / kchunk
  int tpt, mtiles;               // taps per M tile, M tiles
  int nchunks, cps, splits;      // pixel chunks, chunks per split, splits
  int items;                     // mtiles * splits
  int kpad;                      // mtiles * 128
  int stages;                    // TMA ring depth (<= kMaxStages)
  float* partial;                // [splits][kpad][Cout]
  int* err;
};

__device__ __forceinline__ void tma_load_5d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0,
                                            int c1, int c2, int c3, int c4) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%3, %4, %5, %6, %7}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3),
      "r"(c4)
      : "memory");
}

__global__ void __launch_bounds__(kThreads, 1)
    ws_wgrad_tc_kernel(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmD,
                       const WgradParams p) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  unsigned char* base = smem_raw + ((1024 - (raw & 1023)) & 1023);
  const int nst = p.stages;
  const int row_bytes = p.kchunk * 2;                     // 128 or 64: the swizzle span
  const int a_bytes = kTileM * row_bytes;
  const int b_bytes = p.npad * row_bytes;
  const int stage_bytes = ((a_bytes + b_bytes + 1023) / 1024) * 1024;
  SmemCtl* ctl = reinterpret_cast<SmemCtl*>(base + nst * stage_bytes);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < nst; ++s) {
      mbar_init(&ctl->full[s], 1);
      mbar_init(&ctl->empty[s], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&ctl->acc_full[i], 1);
      mbar_init(&ctl->acc_empty[i], 4);
    }
    mbar_init(&ctl->drain, 1);
    ctl->abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&ctl->tmem_base)),
                 "r"(kAccCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = ctl->tmem_base;
  volatile int* abort = &ctl->abort;
  const int ksteps = p.kchunk / 16;
  const uint32_t idesc = instr_desc(kTileM, p.npad);
  const uint32_t acc_stride = 128u;

  if (warp == 4) {
    // ------------------------------------------------ TMA producer
    if (lane == 0) {
      int q = 0, rs = 0, rph = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < p.items && ok; t += gridDim.x) {
        const int mt = t % p.mtiles, sp = t / p.mtiles;
        const int c0 = sp * p.cps, c1 = min(c0 + p.cps, p.nchunks);
        const int tap0 = mt * p.tpt, ntap = min(p.tpt, 9 - tap0);
        const unsigned tx = (unsigned)(ntap * p.Cin * row_bytes + b_bytes);
        for (int c = c0; c < c1 && ok; ++c, ++q, rs = (rs + 1 == nst) ? 0 : rs + 1, rph ^= (rs == 0)) {
          const int s = rs, ph = rph;
          if (!mbar_wait(&ctl->empty[s], ph ^ 1, abort, p.err)) { ok = false; break; }
          const int xt = c % p.xtiles, row = c / p.xtiles;
          const int y = row % p.H, b = row / p.H, x0 = xt * p.kchunk;
          unsigned char* sa = base + s * stage_bytes;
          unsigned char* sb = sa + a_bytes;
          mbar_expect_tx(&ctl->full[s], tx);
          for (int j = 0; j < ntap; ++j) {
            const int tap = tap0 + j, ky = tap / 3, kx = tap % 3;
            tma_load_5d(sa + j * p.Cin * row_bytes, &tmX, &ctl->full[s], x0, y + ky - 1, b, 0, kx);
          }
          tma_load_2d(sb, &tmD, &ctl->full[s], c * p.kchunk, 0);
        }
      }
      if (!ok) {
        for (int k = 0; k < nst; ++k) {
          const int qq = q - 1 - k;
          if (qq < 0) break;
          const int s = qq % nst, ph = (qq / nst) & 1;
          for (unsigned i = 0; i < kSpinLimit && !mbar_try_wait(&ctl->full[s], ph); ++i) {
          }
        }
      }
    }
  } else if (warp == 5) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      int q = 0, rs = 0, rph = 0, local = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < p.items && ok; t += gridDim.x, ++local) {
        const int sp = t / p.mtiles;
        const int c0 = sp * p.cps, c1 = min(c0 + p.cps, p.nchunks);
        const int buf = local & 1, use = local >> 1;
        if (!mbar_wait(&ctl->acc_empty[buf], (use & 1) ^ 1, abort, p.err)) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t d = tmem + buf * acc_stride;
        for (int c = c0; c < c1; ++c, ++q, rs = (rs + 1 == nst) ? 0 : rs + 1, rph ^= (rs == 0)) {
          const int s = rs, ph = rph;
          if (!mbar_wait(&ctl->full[s], ph, abort, p.err)) { ok = false; break; }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t sa = smem_u32(base + s * stage_bytes);
          const uint32_t sb = sa + a_bytes;
          for (int k = 0; k < ksteps; ++k)
            mma_bf16(d, smem_desc(sa + 32 * k, row_bytes), smem_desc(sb + 32 * k, row_bytes), idesc,
                     (c > c0 || k > 0) ? 1u : 0u);
          mma_commit(&ctl->empty[s]);
        }
        if (!ok) break;
        mma_commit(&ctl->acc_full[buf]);
      }
      mma_commit(&ctl->drain);
      for (unsigned i = 0; i < kSpinLimit && !mbar_try_wait(&ctl->drain, 0); ++i) {
      }
    }
  } else {
    // ------------------------------------------------ epilogue (warps 0-3)
    int local = 0;
    const int nvalid = 9 * p.Cin;
    for (int t = blockIdx.x; t < p.items; t += gridDim.x, ++local) {
      const int buf = local & 1, use = local >> 1;
      if (!mbar_wait_warp(&ctl->acc_full[buf], use & 1, abort, p.err)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int mt = t % p.mtiles, sp = t / p.mtiles;
      const int k = mt * kTileM + warp * 32 + lane;          // this lane's row: tap C_in + ci
      float* dst = p.partial + ((size_t)sp * p.kpad + k) * p.Cout;
      const uint32_t tbase = tmem + buf * acc_stride + ((uint32_t)(warp * 32) << 16);
      for (int c0 = 0; c0 < p.npad; c0 += 32) {
        float v[32];
        tmem_ld32(tbase + c0, v);
        if (c0 + 32 >= p.npad) {
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0) mbar_arrive(&ctl->acc_empty[buf]);
        }
        if (k < nvalid) {
          if (c0 + 32 <= p.Cout) {
#pragma unroll
            for (int q4 = 0; q4 < 8; ++q4)
              *reinterpret_cast<float4*>(dst + c0 + 4 * q4) =
                  make_float4(v[4 * q4], v[4 * q4 + 1], v[4 * q4 + 2], v[4 * q4 + 3]);
          } else {
#pragma unroll
            for (int e = 0; e < 32; ++e)
              if (c0 + e < p.Cout) dst[c0 + e] = v[e];
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kAccCols)
                 : "memory");
  }
}

// dW[co][k] = sum over s < splits of partial[s][k][co], in split order;
// consecutive threads take consecutive co, so the partials are read coalesced
__global__ void ws_wgrad_reduce_kernel(int splits, int kpad, int K9, int Cout, const float* __restrict__ part,
                                       float* __restrict__ dW) {
  const long long n = (long long)Cout * K9;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(i / Cout), co = (int)(i % Cout);
    float s = 0.f;
    for (int sp = 0; sp < splits; ++sp) s += part[((size_t)sp * kpad + k) * Cout + co];
    dW[(size_t)co * K9 + k] = s;
  }
}

// XS[s][c][p] = X[p shifted by s - 1 along x][c] (zero past either end of the
// image row) for s < 3 when S = 3; XS[0][c][p] = X[p][c] when S = 1.  X is
// [P][C] bf16 (P = B H W pixels, C <= 128); one block per 128 pixels, staged
// through shared memory as [c][pixel] with a one-pixel halo: 16-byte loads
// (all of a thread's issued before any is stored, so their latencies
// overlap), odd row pitch (the 8 channels of a load land in distinct banks),
// and each warp writes 128 contiguous bytes of one output row at a time.
constexpr int kTrPix = 128;
constexpr int kTrPitch = kTrPix + 3;     // odd
constexpr int kTrBatch = 9;              // 16-byte loads in flight per thread (130 x 16 <= 9 x 256)
__global__ void __launch_bounds__(256) ws_shift_transpose_kernel(long long P, int W, int C, int S, int vec,
                                                                 const __nv_bfloat16* __restrict__ X,
                                                                 __nv_bfloat16* __restrict__ XS) {
  extern __shared__ __nv_bfloat16 tr_s[];          // [C][kTrPitch]: pixel p0 - 1 + i at column i
  const long long p0 = (long long)blockIdx.x * kTrPix;
  constexpr int rows = kTrPix + 2;
  const int tid = threadIdx.x;
  if (vec) {
    const int c8n = C / 8, n = rows * c8n;
    for (int base = 0; base < n; base += kTrBatch * 256) {
      uint4 v[kTrBatch];
#pragma unroll
      for (int r = 0; r < kTrBatch; ++r) {
        const int e = base + tid + 256 * r;
        v[r] = make_uint4(0u, 0u, 0u, 0u);
        if (e < n) {
          const long long pp = p0 - 1 + e / c8n;
          if (pp >= 0 && pp < P) v[r] = __ldg(reinterpret_cast<const uint4*>(X + pp * C + 8 * (e % c8n)));
        }
      }
#pragma unroll
      for (int r = 0; r < kTrBatch; ++r) {
        const int e = base + tid + 256 * r;
        if (e < n) {
          const int i = e / c8n, c = 8 * (e % c8n);
          const __nv_bfloat16* h = reinterpret_cast<const __nv_bfloat16*>(&v[r]);
#pragma unroll
          for (int k = 0; k < 8; ++k) tr_s[(c + k) * kTrPitch + i] = h[k];
        }
      }
    }
  } else {
    const int n = rows * C;
    for (int e = tid; e < n; e += 256) {
      const int i = e / C, c = e % C;
      const long long pp = p0 - 1 + i;
      tr_s[c * kTrPitch + i] = (pp >= 0 && pp < P) ? X[pp * C + c] : __float2bfloat16(0.f);
    }
  }
  __syncthreads();
  const int lane = tid & 31, w = tid >> 5;
  const __nv_bfloat16 z = __float2bfloat16(0.f);
  for (int sc = w; sc < S * C; sc += 8) {
    const int s = sc / C, c = sc % C;
    const int sh = S == 3 ? s - 1 : 0;
    const __nv_bfloat16* row = tr_s + c * kTrPitch;
    __nv_bfloat16* orow = XS + ((size_t)s * C + c) * P;
#pragma unroll
    for (int h = 0; h < kTrPix / 64; ++h) {
      const int i = 2 * lane + 64 * h;             // even pixel offset in the tile
      const long long p = p0 + i;
      if (p >= P) break;
      const int x = (int)(p % W);                  // W even: p and p + 1 share a row
      const int xa = x + sh, xb = x + 1 + sh;
      const __nv_bfloat16 va = (xa >= 0 && xa < W) ? row[i + 1 + sh] : z;
      const __nv_bfloat16 vb = (xb >= 0 && xb < W) ? row[i + 2 + sh] : z;
      if (p + 1 < P) {
        *reinterpret_cast<__nv_bfloat162*>(orow + p) = __halves2bfloat162(va, vb);
      } else {
        orow[p] = va;
      }
    }
  }
}

int sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
  return n > 0 ? n : 1;
}

}  // namespace

// The ring of a CTA with stage_bytes per stage: the deepest ring (up to
// kMaxStages) whose CTA still fits two per SM, or kStages stages at one per
// SM; returns the depth and the dynamic shared memory (stage ring + control
// block + alignment slack).
static int ring_depth(size_t stage_bytes, size_t* smem) {
  const size_t fixed = sizeof(SmemCtl) + 1024;
  int n = PTY_WS_RING_MAX;
  while (n > kStages && n * stage_bytes + fixed > kTwoPerSm) --n;
  const size_t need = n * stage_bytes + fixed;
  *smem = need > kMinSmem ? need : kMinSmem;
  return n;
}

// the largest ring_depth() shared memory of any layer whose stages are at
// most stage_bytes: a deep ring within kTwoPerSm, or kStages stages
static size_t max_ring_smem(size_t stage_bytes) {
  const size_t one = kStages * stage_bytes + sizeof(SmemCtl) + 1024;
  return one > kTwoPerSm ? one : kTwoPerSm;
}

static size_t conv_tc_stage_bytes(int Cin, int Cout) {
  const int chunk = Cin < kChunk ? Cin : kChunk;
  return (((size_t)kTileM * chunk * 2 + (size_t)Cout * chunk * 2 + 1023) / 1024) * 1024;
}

}  // namespace pty

using namespace pty;

static int conv_tc(int32_t B, int32_t H, int32_t W, int32_t Cin, int32_t Cout, const void* X, const void* Wt,
                   const float* bias, int32_t relu, const void* skip, void* out, void* act, float* out32,
                   void* stream);

extern "C" int pty_ws_conv3x3_tc(int32_t B, int32_t H, int32_t W, int32_t Cin, int32_t Cout,
                                 const void* X, const void* Wt, const float* bias, int32_t relu,
                                 const void* skip, void* out, void* act, void* stream) {
  if (!X || !Wt || !bias || !out) return set_error(PTY_ERR_ARG, "pty_ws_conv3x3_tc: null argument");
  return conv_tc(B, H, W, Cin, Cout, X, Wt, bias, relu, skip, out, act, nullptr, stream);
}

extern "C" int pty_ws_conv3x3_tc_f32(int32_t B, int32_t H, int32_t W, int32_t Cin, int32_t Cout, const void* X,
                                     const void* Wt, float* out32, void* stream) {
  if (!X || !Wt || !out32) return set_error(PTY_ERR_ARG, "pty_ws_conv3x3_tc_f32: null argument");
  return conv_tc(B, H, W, Cin, Cout, X, Wt, nullptr, 0, nullptr, nullptr, nullptr, out32, stream);
}

static int conv_tc(int32_t B, int32_t H, int32_t W, int32_t Cin, int32_t Cout, const void* X, const void* Wt,
                   const float* bias, int32_t relu, const void* skip, void* out, void* act, float* out32,
                   void* stream) {
  if (B < 1 || H < 1 || W < 1) return set_error(PTY_ERR_ARG, "pty_ws_conv3x3_tc: empty input");
  if (!(Cin == 32 || Cin % 64 == 0) || Cin > 1024)
    return set_error(PTY_ERR_UNSUPPORTED, "pty_ws_conv3x3_tc: C_in must be 32 or a multiple of 64");
  if (Cout < 32 || Cout > kMaxCout || Cout % 32)
    return set_error(PTY_ERR_UNSUPPORTED, "pty_ws_conv3x3_tc: C_out must be a multiple of 32 in 32..128");
  if (!((W < 128 && 128 % W == 0 && H % (128 / W) == 0) || (W >= 128 && W % 128 == 0)) || W < 8)
    return set_error(PTY_ERR_UNSUPPORTED,
                     "pty_ws_conv3x3_tc: 128-pixel tiles need W dividing 128 (and H a multiple of 128 / W) "
                     "or W a multiple of 128");
  const void* arrays[6] = {X, Wt, out, skip, act, out32};
  for (const void* q : arrays)
    if (q && (reinterpret_cast<uintptr_t>(q) & 15))
      return set_error(PTY_ERR_ARG, "pty_ws_conv3x3_tc: arrays must be 16-byte aligned");
  PFN_cuTensorMapEncodeTiled_v12000 encode;
  PTY_TRY(tensor_map_encoder(&encode));
  int* err = nullptr;
  PTY_TRY(device_timeout_flag(&err));

  ConvParams p{};
  p.B = B; p.H = H; p.W = W; p.Cin = Cin; p.Cout = Cout;
  p.wbox = W < 128 ? W : 128;
  p.rows = 128 / p.wbox;
  p.xtiles = W / p.wbox;
  p.tiles = B * (H / p.rows) * p.xtiles;
  p.chunk_ch = Cin < kChunk ? Cin : kChunk;
  p.chunks = Cin / p.chunk_ch;
  p.relu = relu != 0;
  p.bias = bias;
  p.skip = static_cast<const __nv_bfloat16*>(skip);
  p.out = static_cast<__nv_bfloat16*>(out);
  p.act = static_cast<__nv_bfloat16*>(act);
  p.out32 = out32;
  p.err = err;
  const CUtensorMapSwizzle swz = p.chunk_ch == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B;

  // activations: dims (C, W, H, B), box (chunk, wbox, rows, 1); zero fill outside
  CUtensorMap tmX, tmW;
  {
    const cuuint64_t dims[4] = {(cuuint64_t)Cin, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
    const cuuint64_t strides[3] = {(cuuint64_t)Cin * 2, (cuuint64_t)W * Cin * 2, (cuuint64_t)H * W * Cin * 2};
    const cuuint32_t box[4] = {(cuuint32_t)p.chunk_ch, (cuuint32_t)p.wbox, (cuuint32_t)p.rows, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    CUresult r = encode(&tmX, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(X), dims, strides, box,
                        estr, CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(PTY_ERR_CUDA, "pty_ws_conv3x3_tc: activation tensor map");
  }
  // weights: dims (9 C_in, C_out), box (chunk, C_out)
  {
    const cuuint64_t dims[2] = {(cuuint64_t)9 * Cin, (cuuint64_t)Cout};
    const cuuint64_t strides[1] = {(cuuint64_t)9 * Cin * 2};
    const cuuint32_t box[2] = {(cuuint32_t)p.chunk_ch, (cuuint32_t)Cout};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = encode(&tmW, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(Wt), dims, strides, box,
                        estr, CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(PTY_ERR_CUDA, "pty_ws_conv3x3_tc: weight tensor map");
  }
  size_t smem = 0;
  // halo staging for one-row tiles of 64 input channels whose nine weight
  // taps fit beside a ring of at least two halo stages (C_out <= 64)
  p.halo = (p.rows == 1 && Cin == kChunk && Cout <= 64) ? 1 : 0;
  CUtensorMap tmH;
  if (p.halo) {
    // activations: dims (C, W, H, B), box (64, 130, 1, 1): a tile's input row with one pixel each side
    const cuuint64_t dims[4] = {(cuuint64_t)Cin, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
    const cuuint64_t strides[3] = {(cuuint64_t)Cin * 2, (cuuint64_t)W * Cin * 2, (cuuint64_t)H * W * Cin * 2};
    const cuuint32_t box[4] = {(cuuint32_t)kChunk, (cuuint32_t)kHaloPix, 1, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    CUresult r = encode(&tmH, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(X), dims, strides, box,
                        estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(PTY_ERR_CUDA, "pty_ws_conv3x3_tc: halo tensor map");
    const size_t wtap = (((size_t)Cout * 128 + 1023) / 1024) * 1024;
    const size_t hrow = (((size_t)kHaloPix * 128 + 1023) / 1024) * 1024;
    const size_t fixed = 9 * wtap + sizeof(SmemCtl) + 1024;
    int n = kMaxStages;
    while (n > 2 && n * 3 * hrow + fixed > kHaloSmem) --n;
    p.stages = n;
    smem = n * 3 * hrow + fixed;
  } else {
    p.stages = ring_depth(conv_tc_stage_bytes(Cin, Cout), &smem);
  }
  static std::once_flag attr_once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(attr_once, [] {
    attr_err = cudaFuncSetAttribute(ws_conv_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kHaloSmem);
  });
  if (attr_err != cudaSuccess) return set_cuda_error(attr_err, "pty_ws_conv3x3_tc: smem attribute");
  const int slots = (smem <= kTwoPerSm ? 2 : 1) * sm_count();
  const int grid = p.tiles < slots ? p.tiles : slots;
  ws_conv_tc_kernel<<<grid, kThreads, smem, (cudaStream_t)stream>>>(tmX, tmW, p.halo ? tmH : tmX, p);
  return check_launch("ws_conv_tc_kernel");
}


// ------------------------------------------------------------ weight gradient: host side
namespace pty {
namespace {

struct WgradShape {
  int kchunk, npad, tpt, mtiles, nchunks, cps, splits, kpad;
};

size_t wgrad_stage_bytes(const WgradShape& w) {
  return (((size_t)kTileM * w.kchunk * 2 + (size_t)w.npad * w.kchunk * 2 + 1023) / 1024) * 1024;
}

int wgrad_shape(int B, int H, int W, int Cin, int Cout, WgradShape& w) {
  if (B < 1 || H < 1 || W < 1) return set_error(PTY_ERR_ARG, "pty_ws_wgrad_tc: empty input");
  if (!(Cin == 32 || Cin == 64 || Cin == 128))
    return set_error(PTY_ERR_UNSUPPORTED, "pty_ws_wgrad_tc: C_in must be 32, 64 or 128");
  if (Cout < 1 || Cout > kMaxCout) return set_error(PTY_ERR_UNSUPPORTED, "pty_ws_wgrad_tc: C_out must be 1..128");
  if (!(W == 32 || W % 64 == 0))
    return set_error(PTY_ERR_UNSUPPORTED, "pty_ws_wgrad_tc: W must be 32 or a multiple of 64");
  const long long P = (long long)B * H * W;
  if (P >= (1ll << 31)) return set_error(PTY_ERR_UNSUPPORTED, "pty_ws_wgrad_tc: too many pixels");
  w.kchunk = W == 32 ? 32 : 64;
  w.npad = Cout < 16 ? 16 : ((Cout + 15) / 16) * 16;
  w.tpt = kTileM / Cin;
  w.mtiles = (9 + w.tpt - 1) / w.tpt;
  w.nchunks = (int)(P / w.kchunk);
  // at most two items per CTA slot, every split non-empty
  size_t smem = 0;
  ring_depth(wgrad_stage_bytes(w), &smem);
  const int slots = (smem <= kTwoPerSm ? 2 : 1) * sm_count();
  const int want = 2 * slots / w.mtiles > 0 ? 2 * slots / w.mtiles : 1;
  int splits = want < w.nchunks ? want : w.nchunks;
  w.cps = (w.nchunks + splits - 1) / splits;
  w.splits = (w.nchunks + w.cps - 1) / w.cps;
  w.kpad = w.mtiles * kTileM;
  return PTY_OK;
}


}  // namespace
}  // namespace pty

extern "C" int64_t pty_ws_wgrad_tc_scratch(int32_t B, int32_t H, int32_t W, int32_t Cin, int32_t Cout) {
  WgradShape w;
  if (wgrad_shape(B, H, W, Cin, Cout, w) != PTY_OK) return -1;
  return (int64_t)w.splits * w.kpad * Cout;
}

extern "C" int pty_ws_shift_transpose(int32_t B, int32_t H, int32_t W, int32_t C, int32_t S, const void* X,
                                      void* XS, void* stream) {
  if (B < 1 || H < 1 || W < 2 || (W & 1) || C < 1 || C > 128 || !(S == 1 || S == 3) || !X || !XS)
    return set_error(PTY_ERR_ARG, "pty_ws_shift_transpose: bad arguments");
  if ((reinterpret_cast<uintptr_t>(XS) & 3) != 0)
    return set_error(PTY_ERR_ARG, "pty_ws_shift_transpose: XS must be 4-byte aligned");
  const long long P = (long long)B * H * W;
  const long long blocks = (P + kTrPix - 1) / kTrPix;
  if (blocks >= (1ll << 31)) return set_error(PTY_ERR_UNSUPPORTED, "pty_ws_shift_transpose: too many pixels");
  const size_t smem = (size_t)C * kTrPitch * sizeof(__nv_bfloat16);
  const int vec = C % 8 == 0 && (reinterpret_cast<uintptr_t>(X) & 15) == 0;
  ws_shift_transpose_kernel<<<(unsigned)blocks, 256, smem, (cudaStream_t)stream>>>(
      P, W, C, S, vec, static_cast<const __nv_bfloat16*>(X), static_cast<__nv_bfloat16*>(XS));
  return check_launch("ws_shift_transpose_kernel");
}

extern "C" int pty_ws_wgrad_tc(int32_t B, int32_t H, int32_t W, int32_t Cin, int32_t Cout, const void* XS,
                               const void* dZT, float* dW, float* scratch, int64_t scratch_floats,
                               void* stream) {
  if (!XS || !dZT || !dW || !scratch) return set_error(PTY_ERR_ARG, "pty_ws_wgrad_tc: null argument");
  WgradShape w;
  PTY_TRY(wgrad_shape(B, H, W, Cin, Cout, w));
  if (scratch_floats < (int64_t)w.splits * w.kpad * Cout)
    return set_error(PTY_ERR_ARG, "pty_ws_wgrad_tc: scratch smaller than pty_ws_wgrad_tc_scratch");
  const void* arrays[4] = {XS, dZT, dW, scratch};
  for (const void* q : arrays)
    if (reinterpret_cast<uintptr_t>(q) & 15)
      return set_error(PTY_ERR_ARG, "pty_ws_wgrad_tc: arrays must be 16-byte aligned");
  PFN_cuTensorMapEncodeTiled_v12000 encode;
  PTY_TRY(tensor_map_encoder(&encode));
  int* err = nullptr;
  PTY_TRY(device_timeout_flag(&err));
  const long long P = (long long)B * H * W;
  const CUtensorMapSwizzle swz = w.kchunk == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B;
  CUtensorMap tmX, tmD;
  {
    // XS: dims (W, H, B, C_in, 3 copies), box (chunk, 1, 1, C_in, 1)
    const cuuint64_t dims[5] = {(cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B, (cuuint64_t)Cin, 3};
    const cuuint64_t strides[4] = {(cuuint64_t)W * 2, (cuuint64_t)H * W * 2, (cuuint64_t)P * 2,
                                   (cuuint64_t)Cin * P * 2};
    const cuuint32_t box[5] = {(cuuint32_t)w.kchunk, 1, 1, (cuuint32_t)Cin, 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    CUresult r = encode(&tmX, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(XS), dims, strides, box,
                        estr, CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(PTY_ERR_CUDA, "pty_ws_wgrad_tc: input tensor map");
  }
  {
    // dZT: dims (P, C_out), box (chunk, npad): rows past C_out read zeros
    const cuuint64_t dims[2] = {(cuuint64_t)P, (cuuint64_t)Cout};
    const cuuint64_t strides[1] = {(cuuint64_t)P * 2};
    const cuuint32_t box[2] = {(cuuint32_t)w.kchunk, (cuuint32_t)w.npad};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = encode(&tmD, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(dZT), dims, strides, box,
                        estr, CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(PTY_ERR_CUDA, "pty_ws_wgrad_tc: gradient tensor map");
  }
  WgradParams p{};
  p.B = B; p.H = H; p.W = W; p.Cin = Cin; p.Cout = Cout; p.npad = w.npad;
  p.kchunk = w.kchunk;
  p.xtiles = W / w.kchunk;
  p.tpt = w.tpt; p.mtiles = w.mtiles;
  p.nchunks = w.nchunks; p.cps = w.cps; p.splits = w.splits;
  p.items = w.mtiles * w.splits;
  p.kpad = w.kpad;
  p.partial = scratch;
  p.err = err;
  size_t smem = 0;
  p.stages = ring_depth(wgrad_stage_bytes(w), &smem);
  static std::once_flag attr_once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(attr_once, [] {
    WgradShape big{64, kMaxCout, 1, 9, 1, 1, 1, 9 * kTileM};
    attr_err = cudaFuncSetAttribute(ws_wgrad_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)max_ring_smem(wgrad_stage_bytes(big)));
  });
  if (attr_err != cudaSuccess) return set_cuda_error(attr_err, "pty_ws_wgrad_tc: smem attribute");
  const int slots = (smem <= kTwoPerSm ? 2 : 1) * sm_count();
  const int grid = p.items < slots ? p.items : slots;
  ws_wgrad_tc_kernel<<<grid, kThreads, smem, (cudaStream_t)stream>>>(tmX, tmD, p);
  PTY_TRY(check_launch("ws_wgrad_tc_kernel"));
  const long long n = (long long)Cout * 9 * Cin;
  ws_wgrad_reduce_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(w.splits, w.kpad, 9 * Cin,
                                                                                       Cout, scratch, dW);
  return check_launch("ws_wgrad_reduce_kernel");
}
