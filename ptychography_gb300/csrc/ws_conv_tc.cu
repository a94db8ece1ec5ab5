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
//
// Roles (one CTA per SM, persistent over tiles, 192 threads):
//   warp 4, one lane: TMA producer over a ring of kStages stages;
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
constexpr int kStages = 4;
constexpr int kThreads = 192;
constexpr int kMaxCout = 128;
constexpr int kAccCols = 256;         // TMEM columns: two accumulators of up to 128
// at least this much dynamic shared memory per CTA, so one CTA runs per SM and
// its tensor-memory allocation never waits for another CTA's
constexpr size_t kMinSmem = 116 * 1024;
constexpr unsigned kSpinLimit = 1u << 26;

struct ConvParams {
  int B, H, W, Cin, Cout;
  int wbox, rows;          // input box: wbox pixels x rows image rows (wbox * rows = 128)
  int xtiles;              // tiles per image row (W / 128 when W >= 128, else 1)
  int tiles;               // B * (H / rows) * xtiles
  int chunks;              // ceil(Cin / 64)
  int chunk_ch;            // channels per chunk (64, or Cin when Cin < 64)
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

struct __align__(8) SmemCtl {
  uint64_t full[kStages];
  uint64_t empty[kStages];
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
                      const ConvParams p) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // stage buffers at a 1024-byte boundary (the 128-byte swizzle's atom)
  const uint32_t raw = smem_u32(smem_raw);
  unsigned char* base = smem_raw + ((1024 - (raw & 1023)) & 1023);
  const int a_bytes = kTileM * p.chunk_ch * 2;            // 16 KB (8 KB when C_in = 32)
  const int b_bytes = p.Cout * p.chunk_ch * 2;
  const int stage_bytes = ((a_bytes + b_bytes + 1023) / 1024) * 1024;
  SmemCtl* ctl = reinterpret_cast<SmemCtl*>(base + kStages * stage_bytes);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int swz = p.chunk_ch * 2;                         // 128 or 64 bytes per row

  for (int i = threadIdx.x; i < p.Cout; i += kThreads) ctl->bias[i] = p.bias ? p.bias[i] : 0.f;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
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
  const int ksteps = p.chunk_ch / 16;
  const int nstage_per_tile = 9 * p.chunks;
  const uint32_t idesc = instr_desc(kTileM, p.Cout);
  const uint32_t acc_stride = 128u;                        // column offset of the second accumulator

  if (warp == 4) {
    // ------------------------------------------------ TMA producer
    if (lane == 0) {
      int q = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < p.tiles && ok; t += gridDim.x) {
        int b, y0, x0;
        tile_origin(p, t, b, y0, x0);
        for (int st = 0; st < nstage_per_tile && ok; ++st, ++q) {
          const int s = q % kStages, ph = (q / kStages) & 1;
          if (!mbar_wait(&ctl->empty[s], ph ^ 1, abort, p.err)) { ok = false; break; }
          const int tap = st / p.chunks, ch = st % p.chunks;
          const int ky = tap / 3, kx = tap % 3;
          unsigned char* sa = base + s * stage_bytes;
          unsigned char* sb = sa + a_bytes;
          mbar_expect_tx(&ctl->full[s], (unsigned)(a_bytes + b_bytes));
          tma_load_4d(sa, &tmX, &ctl->full[s], ch * p.chunk_ch, x0 + kx - 1, y0 + ky - 1, b);
          tma_load_2d(sb, &tmW, &ctl->full[s], tap * p.Cin + ch * p.chunk_ch, 0);
        }
      }
      // copies issued but never consumed (after an abort) finish before exit
      if (!ok) {
        for (int k = 0; k < kStages; ++k) {
          const int qq = q - 1 - k;
          if (qq < 0) break;
          const int s = qq % kStages, ph = (qq / kStages) & 1;
          for (unsigned i = 0; i < kSpinLimit && !mbar_try_wait(&ctl->full[s], ph); ++i) {
          }
        }
      }
    }
  } else if (warp == 5) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      int q = 0, local = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < p.tiles && ok; t += gridDim.x, ++local) {
        const int buf = local & 1, use = local >> 1;
        if (!mbar_wait(&ctl->acc_empty[buf], (use & 1) ^ 1, abort, p.err)) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t d = tmem + buf * acc_stride;
        for (int st = 0; st < nstage_per_tile; ++st, ++q) {
          const int s = q % kStages, ph = (q / kStages) & 1;
          if (!mbar_wait(&ctl->full[s], ph, abort, p.err)) { ok = false; break; }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t sa = smem_u32(base + s * stage_bytes);
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
      if (!mbar_wait_warp(&ctl->acc_full[buf], use & 1, abort, p.err)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      int b, y0, x0;
      tile_origin(p, t, b, y0, x0);
      const int r = warp * 32 + lane;                    // pixel row of the tile
      const int y = y0 + r / p.wbox, x = x0 + r % p.wbox;
      const size_t pix = ((size_t)b * p.H + y) * p.W + x;
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
          if (sk) skv = *reinterpret_cast<const uint4*>(sk + 8 * q4);
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

int sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
  return n > 0 ? n : 1;
}

}  // namespace

// dynamic shared memory of one CTA for a layer (stage ring + control block + alignment slack)
static size_t conv_tc_smem(int Cin, int Cout) {
  const int chunk = Cin < kChunk ? Cin : kChunk;
  const size_t stage = (((size_t)kTileM * chunk * 2 + (size_t)Cout * chunk * 2 + 1023) / 1024) * 1024;
  const size_t need = kStages * stage + sizeof(SmemCtl) + 1024;
  return need > kMinSmem ? need : kMinSmem;
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
  const size_t smem = conv_tc_smem(Cin, Cout);
  static std::once_flag attr_once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(attr_once, [] {
    attr_err = cudaFuncSetAttribute(ws_conv_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)conv_tc_smem(64, kMaxCout));
  });
  if (attr_err != cudaSuccess) return set_cuda_error(attr_err, "pty_ws_conv3x3_tc: smem attribute");
  const int grid = p.tiles < sm_count() ? p.tiles : sm_count();
  ws_conv_tc_kernel<<<grid, kThreads, smem, (cudaStream_t)stream>>>(tmX, tmW, p);
  return check_launch("ws_conv_tc_kernel");
}
