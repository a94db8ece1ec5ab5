// 512 x 512 frames on 16-CTA clusters with three-stage line transforms.
//
// The cluster structure of cluster_frame.cuh's (512, 16) tile -- each CTA owns
// 32 rows and 32 columns, rows are pushed to the column owners through
// distributed shared memory, columns run locally, rows are pulled back -- but
// each 512-point line is held by 32 threads x 16 values (line3_fft512,
// 16 x 8 x 4) instead of 16 threads x 32 values, so a CTA runs 512 threads at
// <= 128 registers: 16 warps per SM instead of 8, in ~204 KB of shared memory
// (one CTA per SM):
//   column buffer [512 rows][32 columns] (pitch 32);
//   row scratch: 16 rows in flight x 542 slots -- a row's 32 threads are one
//     warp, so its two exchanges need only __syncwarp();
//   the column pass's first exchange uses the row scratch as [slot][16
//     columns]; its second uses the sub-pass's own column slots, which are
//     dead between the sub-pass's load and its final store (5 CTA barriers
//     per column sub-pass, 2 sub-passes).
// Replaces the same reference functions as frame_kernels.cu.
#include <cooperative_groups.h>

#include "engine.h"
#include "fft_line3.cuh"
#include "frame_ops.cuh"

namespace cg = cooperative_groups;

namespace pty {

namespace {

constexpr int kN = 512, kC = 16, kNT = 512;
constexpr int kA = 32, kB = 16;             // line threads x values
constexpr int kRPC = 32, kRF = 16;          // rows per CTA, rows in flight
constexpr int kCPC = 32, kCW = 16;          // columns per CTA, per column sub-pass
constexpr int kRowScr = 542;                // row-exchange slots (see slot layouts)
constexpr size_t kCbuf = (size_t)kN * kCPC;             // float2
constexpr size_t kRscr = (size_t)kRF * kRowScr;         // float2
constexpr size_t kSmem = (kCbuf + kRscr + kN + 32) * sizeof(float2) + 32 * sizeof(double);
static_assert(kSmem <= 227 * 1024, "shared memory budget");
static_assert((size_t)kRowScr * kCW <= kRscr, "column exchange 1 fits the row scratch");

PTY_DEV void c16_arrive_release() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
PTY_DEV void c16_wait_acquire() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }
PTY_DEV void c16_sync_relaxed() {
  asm volatile("barrier.cluster.arrive.relaxed.aligned;\n\tbarrier.cluster.wait.aligned;" ::: "memory");
}

// Slot layouts (8-byte slots).  Along rows each half-warp touches 16 distinct
// bank pairs: exchange 1 at 34 k1 + t (max 541), exchange 2 at
// (k1 xor 8 (t1 & 1)) + 16 t1 + 64 m1 (max 511).  Along columns a half-warp is
// one line-thread across 16 columns, so any injective layout is
// conflict-free; exchange 2 stays below the column's 512 rows.
PTY_DEV int s1_512(int t, int k1) { return 34 * k1 + t; }
PTY_DEV int s2_512(int k1, int t1, int m1) { return (k1 ^ ((t1 & 1) << 3)) + 16 * t1 + 64 * m1; }

template <int OP>
__global__ void __launch_bounds__(kNT, 1) line3_512_kernel(FrameArgs g) {
  using T = OpTraits<OP>;
  constexpr bool INVERSE = T::INVERSE;
  constexpr float kInv = 1.0f / (float)(kN * kN);

  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int f = blockIdx.x / kC;
  const int tid = threadIdx.x;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* cbuf = reinterpret_cast<float2*>(smem_raw);   // [512][32]
  float2* rscr = cbuf + kCbuf;                            // [16][542] / [542][16]
  float2* tw1 = rscr + kRscr;                             // [16][32]
  float2* tw2 = tw1 + kN;                                 // [8][4]
  double* red = reinterpret_cast<double*>(tw2 + 32);
  for (int i = tid; i < kN; i += kNT) tw1[i] = g.twf[((i & 31) * (i >> 5)) & 511];   // W^(t k1)
  if (tid < 32) tw2[tid] = g.twf[16 * (tid & 3) * (tid >> 2)];                         // W32^(t1 m1)
  int r0 = 0, r1 = 0;
  if (T::IN_EXIT || T::IN_DM) {
    r0 = g.R[2 * f];
    r1 = g.R[2 * f + 1];
  }
  const size_t fbase = (size_t)f * kN * kN;
  float2* psi = g.psi + fbase;
  __syncthreads();

  const int t = tid & 31, lr = tid >> 5;                 // row line: one warp
  float2* rs = rscr + lr * kRowScr;
  auto row_e = [rs](int s) -> float2& { return rs[s]; };
  auto warp_sync = [] { __syncwarp(); };

  // ---------------- row pass: X[a][t + 32 j] belongs to CTA j (local column t)
#pragma unroll 1
  for (int s = 0; s < kRPC / kRF; ++s) {
    const int a = rank * kRPC + s * kRF + lr;
    float2 v[kB];
#pragma unroll
    for (int j = 0; j < kB; ++j) v[j] = frame_input<kN, OP>(g, f, r0, r1, psi, a, t + kA * j);
    line3_fft512<T::FIRST_DIR, true>(v, t, row_e, row_e, s1_512, s2_512, warp_sync, tw1, tw2);
    __syncwarp();                                        // scratch free for the next row
#pragma unroll
    for (int j = 0; j < kB; ++j) cluster.map_shared_rank(cbuf, j)[a * kCPC + t] = v[j];
  }

  const int cw = tid % kCW, tc = tid / kCW;              // column line thread tc < 32
  c16_arrive_release();
  c16_wait_acquire();

  // ---------------- column pass: 2 sub-passes of 16 columns
  ff err = ff_zero();
  auto cta_sync = [] { __syncthreads(); };
#pragma unroll 1
  for (int s = 0; s < kCPC / kCW; ++s) {
    const int cl = s * kCW + cw, kc = rank * kCPC + cl;
    float2 v[kB];
#pragma unroll
    for (int j = 0; j < kB; ++j) v[j] = cbuf[(tc + kA * j) * kCPC + cl];
    auto col_e1 = [rscr, cw](int sl) -> float2& { return rscr[sl * kCW + cw]; };
    auto col_e2 = [cbuf, cl](int sl) -> float2& { return cbuf[sl * kCPC + cl]; };
    line3_fft512<T::FIRST_DIR, false>(v, tc, col_e1, col_e2, s1_512, s2_512, cta_sync, tw1, tw2);
    ModIn<OP, kB> m;
    modulus_load<kN, kN, OP, kA, kB>(g, f, fbase, tc, kc, m);
    modulus_load_late<kN, kN, OP, kA, kB>(g, fbase, tc, kc, m);
    modulus_apply<kN, kN, OP, kA, kB>(g, fbase, tc, kc, v, m, err);
    if constexpr (INVERSE) {
      line3_fft512<+1, false>(v, tc, col_e1, col_e2, s1_512, s2_512, cta_sync, tw1, tw2);
      __syncthreads();                                   // every exchange-2 read done
#pragma unroll
      for (int j = 0; j < kB; ++j) cbuf[(tc + kA * j) * kCPC + cl] = v[j];
    }
  }

  if constexpr (INVERSE) {
    c16_arrive_release();
    c16_wait_acquire();
    // ---------------- inverse row pass, pulled from the column owners
#pragma unroll 1
    for (int s = 0; s < kRPC / kRF; ++s) {
      const int a = rank * kRPC + s * kRF + lr;
      float2 v[kB];
#pragma unroll
      for (int j = 0; j < kB; ++j) v[j] = cluster.map_shared_rank(cbuf, j)[a * kCPC + t];
      line3_fft512<+1, true>(v, t, row_e, row_e, s1_512, s2_512, warp_sync, tw1, tw2);
      __syncwarp();
#pragma unroll
      for (int j = 0; j < kB; ++j) v[j] = cscale(v[j], kInv);
      frame_output_line<kN, OP, kA, kB>(g, r0, r1, psi, a, t, v);
    }
    // every pulled value is consumed before its CTA arrives
    c16_sync_relaxed();
  }

  if (g.err_part) {
    const double sum = block_sum_d(ff_to_double(err), red);
    if (tid == 0) {
      double* ep = g.err_part + (size_t)f * g.err_stride;
      ep[rank] = sum;
      if (rank == 0)
        for (int k = kC; k < g.err_stride; ++k) ep[k] = 0.0;
    }
  }
}

template <int OP>
int set_attr() {
  auto fn = line3_512_kernel<OP>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) return set_cuda_error(e, "line3_512_kernel attributes");
  return PTY_OK;
}

cudaLaunchConfig_t config(int nframes, cudaStream_t st, cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nframes * kC);
  cfg.blockDim = dim3(kNT);
  cfg.dynamicSmemBytes = kSmem;
  cfg.stream = st;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kC;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

template <int OP>
int launch(const FrameArgs& a, int nframes, cudaStream_t st) {
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = config(nframes, st, attr);
  cudaError_t e = cudaLaunchKernelEx(&cfg, line3_512_kernel<OP>, a);
  if (e != cudaSuccess) return set_cuda_error(e, "line3_512_kernel launch");
  return check_launch("line3_512_kernel");
}

}  // namespace

int prepare_cluster_512x16l() {
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
  if (rc) return rc;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = config(1, nullptr, attr);
  int nclusters = 0;
  cudaError_t e = cudaOccupancyMaxActiveClusters(&nclusters, line3_512_kernel<OP_PSI7>, &cfg);
  if (e != cudaSuccess) return set_cuda_error(e, "cudaOccupancyMaxActiveClusters");
  if (nclusters < 1) return set_error(PTY_ERR_UNSUPPORTED, "no 16-CTA cluster of this kernel fits the GPU");
  return PTY_OK;
}

int launch_cluster_512x16l(int op, const FrameArgs& a, int nframes, cudaStream_t st) {
  if (!a.twf) return set_error(PTY_ERR_ARG, "line3_512_kernel needs the full twiddle table");
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
