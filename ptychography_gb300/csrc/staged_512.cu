// 512 x 512 frames in three launches through a frame scratch (tile 264).
//
// A 512^2 complex64 frame (2 MB) fills the shared memory of 16 SMs, so the
// cluster tiles need 16 free SMs of one GPC per frame: on a 152-SM GB300 only
// 7 such clusters are resident at once (112 SMs), whatever the kernel does.
// This tile keeps every SM busy instead, at the price of a scratch round trip:
//   1. row launch: one warp per frame row forms the input wave (exit wave,
//      psi, or the DM combination), row-FFTs it (line3_fft512, warp-local
//      exchanges) and writes the row to the scratch;
//   2. column launch: a CTA takes 8 columns of one frame (32 line threads
//      each), forward column FFT, the modulus constraint, inverse column FFT,
//      and writes the columns back (or, for the forms without an inverse,
//      writes their result);
//   3. row launch: inverse row FFT of the scratch rows, scaled, written as the
//      new wave (with the DM update).
// The scratch holds stage_frames frames; larger launches run group by group.
// Each CTA is independent: no cluster barrier; three row CTAs or two column
// CTAs per SM.  The column launch writes one error partial per CTA: 64 slots
// per frame (the tile id is 200 + 64).
// Line transforms, slot layouts and the per-pixel operations are those of the
// 16-CTA tile 116, so results agree with it to FP32 rounding.
// Replaces the same reference functions as frame_kernels.cu.
#include <cstdint>
#include <cstring>

#include "engine.h"
#include "fft_line3.cuh"
#include "frame_ops.cuh"

namespace pty {

namespace {

constexpr int kN = 512;
constexpr int kA = 32, kB = 16;             // line threads x values
constexpr int kNT = 256;                    // threads per CTA, both launches
constexpr int kRows = kNT / kA;             // rows per row CTA (one warp each)
constexpr int kCols = kNT / kA;             // columns per column CTA
constexpr int kBlocksPerFrame = kN / kRows; // = kN / kCols = 64
constexpr int kRowScr = 542;                // row-exchange slots per warp
constexpr int kColE1 = 527;                 // column exchange-1 slots (33 k1 + t)
// column-launch shared memory, every region at a 128-byte boundary (TMA
// destinations): exchange 1, the scratch columns (then exchange 2), the
// amplitudes, the background, the mask block, the copies' mbarrier
constexpr size_t kAlign128(size_t b) { return (b + 127) / 128 * 128; }
constexpr size_t kOffX2 = kAlign128((size_t)kColE1 * kCols * sizeof(float2));
constexpr size_t kOffA = kOffX2 + (size_t)kN * kCols * sizeof(float2);
constexpr size_t kOffB = kOffA + (size_t)kN * kCols * sizeof(float);
constexpr size_t kOffM = kOffB + (size_t)kN * kCols * sizeof(float);
constexpr size_t kOffBar = kOffM + (size_t)kN * kCols;
constexpr size_t kColSmem = kOffBar + 128 + 128;   // + the barrier, + base alignment slack
constexpr unsigned kSpinLimit = 1u << 26;          // mbarrier polls before giving up
static_assert(kRows == kCols && kBlocksPerFrame == 64, "64 blocks per frame per launch");

// Row slot layouts (a warp is one line; each half-warp touches 16 distinct
// bank pairs): exchange 1 at 34 k1 + t (max 541), exchange 2 at
// (k1 xor 8 (t1 & 1)) + 16 t1 + 64 m1 (max 511).
PTY_DEV int row_s1(int t, int k1) { return 34 * k1 + t; }
PTY_DEV int any_s2(int k1, int t1, int m1) { return (k1 ^ ((t1 & 1) << 3)) + 16 * t1 + 64 * m1; }
// Column slot layouts: slot s of a column sits at s * 8 + column, so a
// half-warp (two line threads x 8 columns) is conflict-free when its two
// slots differ in parity: exchange 1 at 33 k1 + t (max 526); exchange 2 as
// along rows (its two slots differ by one in every access).
PTY_DEV int col_s1(int t, int k1) { return 33 * k1 + t; }

PTY_DEV void load_twiddles(const FrameArgs& g, float2* tw1, float2* tw2) {
  for (int i = threadIdx.x; i < kN; i += kNT) tw1[i] = g.twf[((i & 31) * (i >> 5)) & 511];   // W^(t k1)
  if (threadIdx.x < 32) tw2[threadIdx.x] = g.twf[16 * (threadIdx.x & 3) * (threadIdx.x >> 2)];
}

// Row launch.  !LAST: input wave -> forward row FFT -> scratch.
// LAST: scratch -> inverse row FFT -> scaled output wave.  Three CTAs (24
// warps) per SM: the DM forms, which also read psi and the exit wave, fit in
// 80 registers without spills (at their unconstrained 107-109, two CTAs).
template <int OP, bool LAST>
__global__ void __launch_bounds__(kNT, 3) staged_rows_kernel(FrameArgs g, int f0) {
  using T = OpTraits<OP>;
  constexpr float kInv = 1.0f / (float)(kN * kN);
  __shared__ float2 tw1[kN];
  __shared__ float2 tw2[32];
  __shared__ float2 rscr[kRows * kRowScr];
  load_twiddles(g, tw1, tw2);
  const int fl = blockIdx.x / kBlocksPerFrame, f = f0 + fl;
  const int t = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int a = (blockIdx.x % kBlocksPerFrame) * kRows + w;
  int r0 = 0, r1 = 0;
  if (T::IN_EXIT || T::IN_DM) {
    r0 = g.R[2 * f];
    r1 = g.R[2 * f + 1];
  }
  float2* psi = g.psi + (size_t)f * kN * kN;
  float2* srow = g.stage + (size_t)fl * kN * kN + (size_t)a * kN;
  float2* rs = rscr + w * kRowScr;
  auto row_e = [rs](int s) -> float2& { return rs[s]; };
  auto warp_sync = [] { __syncwarp(); };
  __syncthreads();
  float2 v[kB];
  if constexpr (!LAST) {
#pragma unroll
    for (int j = 0; j < kB; ++j) v[j] = frame_input<kN, OP>(g, f, r0, r1, psi, a, t + kA * j);
    line3_fft512<T::FIRST_DIR, true>(v, t, row_e, row_e, row_s1, any_s2, warp_sync, tw1, tw2);
#pragma unroll
    for (int j = 0; j < kB; ++j) srow[t + kA * j] = v[j];
  } else {
#pragma unroll
    for (int j = 0; j < kB; ++j) v[j] = srow[t + kA * j];
    line3_fft512<+1, true>(v, t, row_e, row_e, row_s1, any_s2, warp_sync, tw1, tw2);
#pragma unroll
    for (int j = 0; j < kB; ++j) v[j] = cscale(v[j], kInv);
    frame_output_line<kN, OP, kA, kB>(g, r0, r1, psi, a, t, v);
  }
}

PTY_DEV uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
PTY_DEV void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
PTY_DEV bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// 2-D box of a 3-D tensor map (columns, rows, frames) into shared memory
PTY_DEV void tma_box(void* dst, const CUtensorMap* map, uint64_t* bar, int c, int r, int f) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_addr(bar)), "r"(c), "r"(r), "r"(f)
      : "memory");
}
// contiguous bytes (a multiple of 16, both addresses 16-byte aligned)
PTY_DEV void bulk_copy(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// The column launch's tensor maps: boxes of 8 columns x 256 rows of one frame
struct ColMaps {
  CUtensorMap stage;   // the frame scratch (8-byte elements: complex64)
  CUtensorMap amp;     // amplitudes
  CUtensorMap bg;      // the background the operation reads
};

// The mask in column-block order for the column launch:
// blk[b][r][c] = mask[r][8 b + c] (64 blocks of 512 rows x 8 columns).
__global__ void __launch_bounds__(kNT) mask_blocks_kernel(const uint8_t* __restrict__ mask,
                                                          uint8_t* __restrict__ blk) {
  const int b = blockIdx.x;
  for (int i = threadIdx.x; i < kN * kCols; i += kNT) {
    const int r = i / kCols, c = i % kCols;
    blk[(size_t)b * kN * kCols + i] = mask[(size_t)r * kN + kCols * b + c];
  }
}

// Column launch: 8 columns of one frame per CTA, thread (cw, tc) = line
// thread tc of column c0 + cw.  Every global input of the CTA -- its scratch
// columns, amplitudes and background -- is copied into shared memory by TMA
// at the start, with its block of the mask (shared by all frames,
// L2-resident), so the CTA waits for memory once and holds no registers for
// loads in flight.
template <int OP>
__global__ void __launch_bounds__(kNT, 2) staged_cols_kernel(FrameArgs g, int f0, const __grid_constant__ ColMaps maps,
                                                              int amp_frames, int bg_frames) {
  using T = OpTraits<OP>;
  using MI = ModIn<OP, kB>;
  __shared__ float2 tw1[kN];
  __shared__ float2 tw2[32];
  __shared__ double red[32];
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* base = smem_raw + ((128 - (smem_addr(smem_raw) & 127)) & 127);
  float2* x1 = reinterpret_cast<float2*>(base);                // [527][8] exchange 1
  float2* x2 = reinterpret_cast<float2*>(base + kOffX2);       // [512][8] input, then exchange 2
  float* sa = reinterpret_cast<float*>(base + kOffA);          // [512][8] amplitudes
  float* sb = reinterpret_cast<float*>(base + kOffB);          // [512][8] background (or DM state)
  uint8_t* sm = base + kOffM;                                  // [512][8] mask
  uint64_t* bar = reinterpret_cast<uint64_t*>(base + kOffBar);
  const int fl = blockIdx.x / kBlocksPerFrame, f = f0 + fl;
  const int blk = blockIdx.x % kBlocksPerFrame;
  const int cw = threadIdx.x % kCols, tc = threadIdx.x / kCols;
  const int kc = blk * kCols + cw;
  const size_t fbase = (size_t)f * kN * kN;
  float2* scol = g.stage + (size_t)fl * kN * kN + kc;
  constexpr bool BG_ST = MI::BG_IN || OP == OP_DM7;
  const float* bsrc = nullptr;
  if constexpr (MI::BG_IN) bsrc = g.bg_in ? g.bg_in + (size_t)g.bg_stride * f : nullptr;
  if constexpr (OP == OP_DM7) bsrc = g.bg_out + fbase;
  // Every global input of the CTA -- its 8 scratch columns, amplitudes and
  // background (two 8 x 256 boxes each) and its 4 KB block of the mask --
  // arrives by TMA on one mbarrier: 8 copies instead of ~8000 16-byte
  // requests, no registers held for loads in flight.
  const int c0 = blk * kCols;
  const bool want_bg = BG_ST && bsrc != nullptr;
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    unsigned bytes = 2u * 256u * kCols * sizeof(float2);
    if constexpr (MI::NEEDS) {
      bytes += 2u * 256u * kCols * sizeof(float);
      if (g.mask) bytes += kN * kCols;
    }
    if (want_bg) bytes += 2u * 256u * kCols * sizeof(float);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
    for (int h = 0; h < 2; ++h) tma_box(x2 + h * 256 * kCols, &maps.stage, bar, c0, 256 * h, fl);
    if constexpr (MI::NEEDS) {
      const int af = amp_frames > 1 ? f : 0;
      for (int h = 0; h < 2; ++h) tma_box(sa + h * 256 * kCols, &maps.amp, bar, c0, 256 * h, af);
      // the mask's column-block copy: this CTA's 512 rows x 8 columns in one piece
      if (g.mask) bulk_copy(sm, g.mask_blk + (size_t)blk * kN * kCols, kN * kCols, bar);
    }
    if (want_bg) {
      const int bf = bg_frames > 1 ? f : 0;
      for (int h = 0; h < 2; ++h) tma_box(sb + h * 256 * kCols, &maps.bg, bar, c0, 256 * h, bf);
    }
  }
  __syncthreads();   // the barrier's initialisation before anyone polls it
  load_twiddles(g, tw1, tw2);
  auto e1 = [x1, cw](int s) -> float2& { return x1[s * kCols + cw]; };
  auto e2 = [x2, cw](int s) -> float2& { return x2[s * kCols + cw]; };
  auto cta_sync = [] { __syncthreads(); };
  {
    // bounded wait: past the limit the flag is set and the CTA only waits
    // (again bounded) for its copies before returning
    bool ok = false;
    for (unsigned i = 0; i < kSpinLimit && !ok; ++i) ok = mbar_try_wait(bar, 0);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0 && g.timeout) atomicExch(g.timeout, 1);
      for (unsigned i = 0; i < kSpinLimit && !mbar_try_wait(bar, 0); ++i) {
      }
      return;
    }
  }
  float2 v[kB];
  // the transform's first barrier orders these reads before exchange 2
  // overwrites x2
#pragma unroll
  for (int j = 0; j < kB; ++j) v[j] = x2[(tc + kA * j) * kCols + cw];
  line3_fft512<T::FIRST_DIR, false>(v, tc, e1, e2, col_s1, any_s2, cta_sync, tw1, tw2);
  ff err = ff_zero();
  if constexpr (MI::NEEDS) {
    MI m;
#pragma unroll
    for (int j = 0; j < kB; ++j) {
      const int r = tc + kA * j, sl = r * kCols + cw;
      m.am[j] = sa[sl];
      m.mk[j] = g.mask ? byte_to_float(sm[sl]) : 1.0f;
      if constexpr (BG_ST) m.bb[j] = bsrc ? sb[sl] : 0.0f;
      if constexpr (OP == OP_DM7) m.b0v[j] = __ldg(&g.b0[(size_t)r * kN + kc]);
    }
    modulus_compute<OP, kB>(g, v, m, err);
    if constexpr (MI::BG_OUT) {
#pragma unroll
      for (int j = 0; j < kB; ++j) g.bg_out[fbase + (size_t)(tc + kA * j) * kN + kc] = m.bb[j];
    }
  } else {
    MI m;
    modulus_apply<kN, kN, OP, kA, kB>(g, fbase, tc, kc, v, m, err);
  }
  if constexpr (T::INVERSE) {
    line3_fft512<+1, false>(v, tc, e1, e2, col_s1, any_s2, cta_sync, tw1, tw2);
#pragma unroll
    for (int j = 0; j < kB; ++j) scol[(size_t)(tc + kA * j) * kN] = v[j];
  }
  if (g.err_part) {
    const double sum = block_sum_d(ff_to_double(err), red);
    if (threadIdx.x == 0) {
      double* ep = g.err_part + (size_t)f * g.err_stride;
      ep[blk] = sum;
      if (blk == 0)
        for (int k = kBlocksPerFrame; k < g.err_stride; ++k) ep[k] = 0.0;
    }
  }
}

template <int OP>
int set_attr() {
  cudaError_t e = cudaFuncSetAttribute(staged_cols_kernel<OP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kColSmem);
  if (e != cudaSuccess) return set_cuda_error(e, "staged_cols_kernel attributes");
  return PTY_OK;
}

// A 3-D tensor map (columns, rows, frames) over 512 x 512 frames of `esize`
// bytes per element, frames `fstride` elements apart (0: one shared frame),
// with 8 x 256 boxes.
int frame_map(CUtensorMap* m, const void* base, CUtensorMapDataType type, int esize, long long fstride,
              int frames) {
  PFN_cuTensorMapEncodeTiled_v12000 encode;
  PTY_TRY(tensor_map_encoder(&encode));
  const bool shared = fstride == 0;
  const cuuint64_t dims[3] = {(cuuint64_t)kN, (cuuint64_t)kN, (cuuint64_t)(shared ? 1 : frames)};
  const cuuint64_t strides[2] = {(cuuint64_t)kN * esize,
                                 (cuuint64_t)(shared ? (long long)kN * kN : fstride) * esize};
  const cuuint32_t box[3] = {(cuuint32_t)kCols, 256, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = encode(m, type, 3, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                      CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(PTY_ERR_CUDA, "staged frame tile: tensor map");
  return PTY_OK;
}

template <int OP>
int launch(const FrameArgs& a, int nframes, cudaStream_t st) {
  using MI = ModIn<OP, kB>;
  ColMaps maps;
  std::memset(&maps, 0, sizeof(maps));
  PTY_TRY(frame_map(&maps.stage, a.stage, CU_TENSOR_MAP_DATA_TYPE_UINT64, 8, (long long)kN * kN, a.stage_frames));
  int amp_frames = 1, bg_frames = 1;
  if (MI::NEEDS) {
    amp_frames = a.amp_stride ? nframes : 1;
    PTY_TRY(frame_map(&maps.amp, a.amp, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, a.amp_stride, nframes));
  }
  if (MI::BG_IN && a.bg_in) {
    bg_frames = a.bg_stride ? nframes : 1;
    PTY_TRY(frame_map(&maps.bg, a.bg_in, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, a.bg_stride, nframes));
  } else if (OP == OP_DM7) {
    bg_frames = nframes;
    PTY_TRY(frame_map(&maps.bg, a.bg_out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, (long long)kN * kN, nframes));
  }
  if (a.mask) {
    mask_blocks_kernel<<<kBlocksPerFrame, kNT, 0, st>>>(a.mask, a.mask_blk);
    PTY_TRY(check_launch("mask_blocks_kernel"));
  }
  for (int f0 = 0; f0 < nframes; f0 += a.stage_frames) {
    const int nf = nframes - f0 < a.stage_frames ? nframes - f0 : a.stage_frames;
    const dim3 grid(nf * kBlocksPerFrame);
    staged_rows_kernel<OP, false><<<grid, kNT, 0, st>>>(a, f0);
    PTY_TRY(check_launch("staged_rows_kernel"));
    staged_cols_kernel<OP><<<grid, kNT, kColSmem, st>>>(a, f0, maps, amp_frames, bg_frames);
    PTY_TRY(check_launch("staged_cols_kernel"));
    if constexpr (OpTraits<OP>::INVERSE) {
      staged_rows_kernel<OP, true><<<grid, kNT, 0, st>>>(a, f0);
      PTY_TRY(check_launch("staged_rows_kernel"));
    }
  }
  return PTY_OK;
}

}  // namespace

int prepare_staged_512() {
  int rc = PTY_OK;
  if (!rc) rc = set_attr<OP_EXIT1>();
  if (!rc) rc = set_attr<OP_EXIT7>();
  if (!rc) rc = set_attr<OP_PSI1>();
  if (!rc) rc = set_attr<OP_PSI7>();
  if (!rc) rc = set_attr<OP_DM1>();
  if (!rc) rc = set_attr<OP_DM7>();
  if (!rc) rc = set_attr<OP_MERR>();
  if (!rc) rc = set_attr<OP_INTENS>();
  if (!rc) rc = set_attr<OP_MERR_PSI>();
  if (!rc) rc = set_attr<OP_BP>();
  return rc;
}

int launch_staged_512(int op, const FrameArgs& a, int nframes, cudaStream_t st) {
  if (!a.twf) return set_error(PTY_ERR_ARG, "staged frame tile needs the full twiddle table");
  if (!a.stage || a.stage_frames < 1 || (a.mask && !a.mask_blk))
    return set_error(PTY_ERR_ARG, "staged frame tile needs its frame and mask scratch");
  if (a.err_part && a.err_stride < kBlocksPerFrame)
    return set_error(PTY_ERR_ARG, "staged frame tile needs 64 error slots per frame");
  // the column launch copies amplitude and background rows in 16-byte
  // pieces; arrays not 16-byte aligned go through the 16-CTA tile with the
  // same line transforms instead (same waves and background, error partials
  // grouped per 16 CTAs)
  auto misaligned = [](const void* q, uintptr_t m) { return ((uintptr_t)q & m) != 0; };
  if (misaligned(a.amp, 15) || misaligned(a.bg_in, 15) || misaligned(a.bg_out, 15)) {
    PTY_TRY(prepare_cluster_512x16l());
    return launch_cluster_512x16l(op, a, nframes, st);
  }
  switch (op) {
    case OP_EXIT1: return launch<OP_EXIT1>(a, nframes, st);
    case OP_EXIT7: return launch<OP_EXIT7>(a, nframes, st);
    case OP_PSI1: return launch<OP_PSI1>(a, nframes, st);
    case OP_PSI7: return launch<OP_PSI7>(a, nframes, st);
    case OP_DM1: return launch<OP_DM1>(a, nframes, st);
    case OP_DM7: return launch<OP_DM7>(a, nframes, st);
    case OP_MERR: return launch<OP_MERR>(a, nframes, st);
    case OP_INTENS: return launch<OP_INTENS>(a, nframes, st);
    case OP_MERR_PSI: return launch<OP_MERR_PSI>(a, nframes, st);
    case OP_BP: return launch<OP_BP>(a, nframes, st);
  }
  return set_error(PTY_ERR_ARG, "unknown frame op");
}

}  // namespace pty
