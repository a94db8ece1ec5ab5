// 256 x 256 frames on 8-CTA clusters with three-stage line transforms.
//
// The same cluster structure as cluster_frame.cuh's (256, 8) tile -- each CTA
// owns 32 rows and 32 columns, rows are pushed to the column owners through
// distributed shared memory, columns run locally, rows are pulled back -- but
// each 256-point line is held by 32 threads x 8 values (fft_line3.cuh) instead
// of 16 x 16, so a CTA runs 512 threads at <= 64 registers and two CTAs (32
// warps) share an SM within the same ~108 KB of shared memory per CTA:
//   column buffer [256 rows][32 columns] (pitch 32);
//   row scratch: 16 rows in flight x 312 slots -- a row's 32 threads are one
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

constexpr int kN = 256, kC = 8, kNT = 512;
constexpr int kA = 32, kB = 8;              // line threads x values
constexpr int kRPC = 32, kRF = 16;          // rows per CTA, rows in flight
constexpr int kCPC = 32, kCW = 16;          // columns per CTA, per column sub-pass
constexpr int kRowScr = 312;                // row-exchange slots (see slot layouts)
constexpr size_t kCbuf = (size_t)kN * kCPC;             // float2
constexpr size_t kRscr = (size_t)kRF * kRowScr;         // float2
constexpr size_t kSmem = (kCbuf + kRscr + 2 * (size_t)kN) * sizeof(float2) + 32 * sizeof(double);
static_assert(kSmem + 1024 <= 114 * 1024, "two CTAs per SM");
static_assert((size_t)270 * kCW <= kRscr, "column exchange 1 fits the row scratch");

PTY_DEV void l3_arrive_release() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
PTY_DEV void l3_wait_acquire() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }
PTY_DEV void l3_sync_relaxed() {
  asm volatile("barrier.cluster.arrive.relaxed.aligned;\n\tbarrier.cluster.wait.aligned;" ::: "memory");
}

// Row slot layouts (8-byte slots; each half-warp touches 16 distinct bank pairs):
//   exchange 1 at 34 k1 + t, exchange 2 at k1 + 8 t1 + 40 m1 (max 311).
PTY_DEV int row_s1(int t, int k1) { return 34 * k1 + t; }
PTY_DEV int row_s2(int k1, int t1, int m1) { return k1 + 8 * t1 + 40 * m1; }
// Column slot layouts: a half-warp is one line-thread across 16 columns, so
// any injective layout is conflict-free; exchange 2 must stay below 256 rows.
PTY_DEV int col_s1(int t, int k1) { return 34 * k1 + t; }        // < 270
PTY_DEV int col_s2(int k1, int t1, int m1) { return k1 + 8 * t1 + 32 * m1; }   // < 256

template <int OP>
__global__ void __launch_bounds__(kNT, 2) line3_cluster_kernel(FrameArgs g) {
  using T = OpTraits<OP>;
  constexpr bool INVERSE = T::INVERSE;
  constexpr float kInv = 1.0f / (float)(kN * kN);

  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int f = blockIdx.x / kC;
  const int tid = threadIdx.x;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* cbuf = reinterpret_cast<float2*>(smem_raw);   // [256][32]
  float2* rscr = cbuf + kCbuf;                            // [16][312] / [270][16]
  float2* tw1 = rscr + kRscr;                             // [8][32]
  float2* twf = tw1 + kN;                                 // [256]
  double* red = reinterpret_cast<double*>(twf + kN);
  for (int i = tid; i < kN; i += kNT) {
    twf[i] = g.twf[i];
    tw1[i] = g.twf[((i & 31) * (i >> 5)) & 255];          // tw1[k1 * 32 + t] = W^(t k1)
  }
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
    line3_fft256<T::FIRST_DIR, true>(v, t, row_e, row_e, row_s1, row_s2, warp_sync, tw1, twf);
    __syncwarp();                                        // scratch free for the next row
#pragma unroll
    for (int j = 0; j < kB; ++j) cluster.map_shared_rank(cbuf, j)[a * kCPC + t] = v[j];
  }

  const int cw = tid % kCW, tc = tid / kCW;              // column line thread tc < 32
  l3_arrive_release();
  l3_wait_acquire();

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
    line3_fft256<T::FIRST_DIR, false>(v, tc, col_e1, col_e2, col_s1, col_s2, cta_sync, tw1, twf);
    // the modulus inputs are loaded here, after the transform: at 64 registers
    // they cannot be held across it (32 warps per SM cover the latency instead)
    ModIn<OP, kB> m;
    modulus_load<kN, kN, OP, kA, kB>(g, f, fbase, tc, kc, m);
    modulus_load_late<kN, kN, OP, kA, kB>(g, fbase, tc, kc, m);
    modulus_apply<kN, kN, OP, kA, kB>(g, fbase, tc, kc, v, m, err);
    if constexpr (INVERSE) {
      line3_fft256<+1, false>(v, tc, col_e1, col_e2, col_s1, col_s2, cta_sync, tw1, twf);
      __syncthreads();                                   // every exchange-2 read done
#pragma unroll
      for (int j = 0; j < kB; ++j) cbuf[(tc + kA * j) * kCPC + cl] = v[j];
    }
  }

  if constexpr (INVERSE) {
    l3_arrive_release();
    l3_wait_acquire();
    // ---------------- inverse row pass, pulled from the column owners
#pragma unroll 1
    for (int s = 0; s < kRPC / kRF; ++s) {
      const int a = rank * kRPC + s * kRF + lr;
      float2 v[kB];
#pragma unroll
      for (int j = 0; j < kB; ++j) v[j] = cluster.map_shared_rank(cbuf, j)[a * kCPC + t];
      line3_fft256<+1, true>(v, t, row_e, row_e, row_s1, row_s2, warp_sync, tw1, twf);
      __syncwarp();
#pragma unroll
      for (int j = 0; j < kB; ++j) v[j] = cscale(v[j], kInv);
      frame_output_line<kN, OP, kA, kB>(g, r0, r1, psi, a, t, v);
    }
    // every pulled value is consumed before its CTA arrives
    l3_sync_relaxed();
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
  cudaError_t e = cudaFuncSetAttribute(line3_cluster_kernel<OP>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
  if (e != cudaSuccess) return set_cuda_error(e, "line3_cluster_kernel attributes");
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
  cudaError_t e = cudaLaunchKernelEx(&cfg, line3_cluster_kernel<OP>, a);
  if (e != cudaSuccess) return set_cuda_error(e, "line3_cluster_kernel launch");
  return check_launch("line3_cluster_kernel");
}

}  // namespace

int prepare_cluster_256x8l() {
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
  cudaError_t e = cudaOccupancyMaxActiveClusters(&nclusters, line3_cluster_kernel<OP_PSI7>, &cfg);
  if (e != cudaSuccess) return set_cuda_error(e, "cudaOccupancyMaxActiveClusters");
  if (nclusters < 1) return set_error(PTY_ERR_UNSUPPORTED, "no 8-CTA cluster of this kernel fits the GPU");
  return PTY_OK;
}

int launch_cluster_256x8l(int op, const FrameArgs& a, int nframes, cudaStream_t st) {
  if (!a.twf) return set_error(PTY_ERR_ARG, "line3_cluster_kernel needs the full twiddle table");
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
