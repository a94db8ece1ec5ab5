// Square frames on thread-block clusters: one frame per cluster of C CTAs.
//
// A 256^2 complex64 frame (512 KB) or 512^2 frame (2 MB) does not fit one SM's
// shared memory, so the 2-D transform is distributed over a cluster of C CTAs,
// each owning N / C rows and N / C columns, and the two transposes go through
// distributed shared memory instead of HBM.  The frame tiles built (N, C):
// (128, 2), (192, 2), (256, 4), (256, 8), (512, 16); each is instantiated in
// its own translation unit (cluster_<N>x<C>.cu) and chosen per frame size by
// the tile autotuner (frame_tiles.cu).  Per frame (64 rows per CTA shown for
// 256^2 on 4 CTAs):
//
//   1. CTA r forms its 64 rows of the input wave (exit wave, psi, or the DM
//      combination), row-FFTs them, and stores each transformed row straight
//      into the column buffer of the CTA that owns those 64 columns
//      (remote st.shared::cluster through map_shared_rank);
//   2. cluster barrier;
//   3. CTA r runs its 64 columns entirely locally: forward column FFT, the
//      modulus constraint in registers, inverse column FFT, in place;
//   4. cluster barrier;
//   5. CTA r pulls its 64 rows back from the four column buffers, inverse
//      row-FFTs them and writes the result to HBM;
//   6. cluster barrier (no CTA leaves while others still read its buffer).
//
// HBM sees only the frame's input and output (plus the L2-resident object
// window and probe), the same traffic as the single-CTA kernel for small frames.
// Replaces the same reference functions as frame_kernels.cu.
#pragma once
#include <cooperative_groups.h>

#include "engine.h"
#include "fft_line.cuh"
#include "frame_ops.cuh"

namespace cg = cooperative_groups;

namespace pty {

// Cluster barrier without memory ordering: used only to keep every CTA's
// shared memory alive until the others have finished reading it, which needs
// no release of this CTA's own (global) stores.
PTY_DEV void cluster_sync_relaxed() {
  asm volatile("barrier.cluster.arrive.relaxed.aligned;\n\tbarrier.cluster.wait.aligned;" ::: "memory");
}
// The two halves of a cluster barrier with release / acquire ordering, so that
// independent work (global loads) can be issued between arrival and wait.
PTY_DEV void cluster_arrive_release() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
PTY_DEV void cluster_wait_acquire() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

template <int N, int C>
struct ClusterCfg {
  static constexpr int A = LineGeom<N>::A, B = LineGeom<N>::B;  // rows and columns alike
  // 256 threads per CTA for 8- and 16-CTA clusters and frames up to 192^2
  // (two CTAs per SM where the shared memory allows), else 512
  static constexpr int NT = (C >= 8 || N <= 192) ? 256 : 512;
  static constexpr int RPC = N / C;          // rows owned per CTA
  static constexpr int CPC = N / C;          // columns owned per CTA
  static constexpr int CP = CPC + 1;         // column-buffer pitch (float2), odd
  static constexpr int RF = NT / A;          // rows in flight per row sub-pass
  static constexpr int ROWLEN = B * (A + 1); // padded row-exchange length
  static constexpr int CW = NT / A;          // columns per column sub-pass
  static constexpr int JPC = CPC / A;        // row registers per destination CTA
  static constexpr size_t CBUF = (size_t)N * CP + N / A;  // + one skew slot per A rows
  static constexpr size_t RSCR = (size_t)RF * ROWLEN;
  static constexpr size_t SMEM = (CBUF + RSCR + N) * sizeof(float2) + 32 * sizeof(double);
  static_assert(RPC % RF == 0 && CPC % CW == 0 && CPC % A == 0 && CW >= 8, "cluster split");
  static_assert(SMEM <= 227 * 1024, "shared memory budget");
  // the column pass exchanges through the (then idle) row scratch
  static_assert((size_t)N * CW <= RSCR, "column exchange fits the row scratch");
  // CTAs per SM the shared-memory budget allows (1 KB per CTA reserved by the system)
  static constexpr int MINB_SMEM = (int)((228 * 1024) / (SMEM + 1024));
  static constexpr int MINB = MINB_SMEM > 4 ? 4 : (MINB_SMEM < 1 ? 1 : MINB_SMEM);
};

template <int N, int C, int OP>
__global__ void __launch_bounds__(ClusterCfg<N, C>::NT, ClusterCfg<N, C>::MINB)
    cluster_frame_kernel(FrameArgs g) {
  using K = ClusterCfg<N, C>;
  constexpr int A = K::A, B = K::B, CP = K::CP, RPC = K::RPC, CPC = K::CPC, RF = K::RF, CW = K::CW;
  constexpr int JPC = K::JPC;
  constexpr bool INVERSE = OpTraits<OP>::INVERSE;
  constexpr float kInv = 1.0f / (float)(N * N);

  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int f = blockIdx.x / C;
  const int tid = threadIdx.x;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* cbuf = reinterpret_cast<float2*>(smem_raw);   // [N rows][CPC own columns]
  float2* rscr = cbuf + K::CBUF;                          // [RF][ROWLEN] row exchange
  float2* tw = rscr + K::RSCR;                            // [N]
  double* red = reinterpret_cast<double*>(tw + N);
  for (int i = tid; i < N; i += K::NT) tw[i] = g.tw0[i];

  // Column buffer: element (row r, owned column cl) at r * CP + cl + r / A.
  // With CP odd and the skew of one slot per A rows, both the natural walk
  // (rows t + A j) and the exchange walk (rows A t + tt) of the A lanes of a
  // column land in distinct banks.
  auto cidx = [](int r, int cl) { return r * CP + cl + r / A; };
  // column buffer of cluster rank q (q is a compile-time constant at every use)
  auto rc = [&](int q) { return cluster.map_shared_rank(cbuf, q); };

  int r0 = 0, r1 = 0;
  if (OpTraits<OP>::IN_EXIT || OpTraits<OP>::IN_DM) {
    r0 = g.R[2 * f];
    r1 = g.R[2 * f + 1];
  }
  const size_t fbase = (size_t)f * N * N;
  float2* psi = g.psi + fbase;
  __syncthreads();

  const int t = tid % A, lr = tid / A;
  float2* rs = rscr + lr * K::ROWLEN;

  // ---------------- 1. forward row pass, pushed to the column owners
#pragma unroll 1
  for (int s = 0; s < RPC / RF; ++s) {
    const int a = rank * RPC + s * RF + lr;
    float2 v[B];
#pragma unroll
    for (int j = 0; j < B; ++j) v[j] = frame_input<N, OP>(g, f, r0, r1, psi, a, t + A * j);
    line_stage1<N, OpTraits<OP>::FIRST_DIR>(v, t, tw);
    __syncwarp();
#pragma unroll
    for (int k1 = 0; k1 < B; ++k1) rs[k1 * (A + 1) + t] = v[k1];
    __syncwarp();
    line_stage2<N, OpTraits<OP>::FIRST_DIR>(v, t, [&](int tt, int k1) { return rs[k1 * (A + 1) + tt]; });
    // v[j] = X[a][t + A j]; column t + A j belongs to CTA j / JPC
#pragma unroll
    for (int j = 0; j < B; ++j) rc(j / JPC)[cidx(a, t + A * (j % JPC))] = v[j];
  }
  // the modulus inputs of the first column sub-pass are loaded while the
  // cluster barrier completes
  ModIn<OP, B> m;
  cluster_arrive_release();
  modulus_load<N, N, OP, A, B>(g, f, fbase, tid / CW, rank * CPC + tid % CW, m);
  cluster_wait_acquire();

  // ---------------- 3. column pass on the owned columns
  // Lanes of a warp run along a row (coalesced amp / mask / background
  // traffic); the A threads of a column sit in A different warps.  The
  // exchanges go through the row scratch, idle during this pass, as a
  // [row slot][CW columns] array, so loads of the column buffer and exchange
  // writes never collide and fewer CTA barriers are needed.
  ff err = ff_zero();
  float2* xb = rscr;
#pragma unroll 1
  for (int s = 0; s < CPC / CW; ++s) {
    const int cw = tid % CW, tc = tid / CW;
    const int cl = s * CW + cw;
    const int kc = rank * CPC + cl;
    // this sub-pass's amp / mask / background, in flight during the forward FFT
    if (s > 0) modulus_load<N, N, OP, A, B>(g, f, fbase, tc, kc, m);
    float2 v[B];
#pragma unroll
    for (int j = 0; j < B; ++j) v[j] = cbuf[cidx(tc + A * j, cl)];
    line_stage1<N, OpTraits<OP>::FIRST_DIR>(v, tc, tw);
    if (s > 0) __syncthreads();   // previous sub-pass done reading xb
#pragma unroll
    for (int k1 = 0; k1 < B; ++k1) xb[(k1 * A + tc) * CW + cw] = v[k1];
    __syncthreads();
    line_stage2<N, OpTraits<OP>::FIRST_DIR>(v, tc, [&](int tt, int k1) { return xb[(k1 * A + tt) * CW + cw]; });
    modulus_load_late<N, N, OP, A, B>(g, fbase, tc, kc, m);
    modulus_apply<N, N, OP, A, B>(g, fbase, tc, kc, v, m, err);
    if constexpr (INVERSE) {
      line_stage1<N, +1>(v, tc, tw);
      __syncthreads();
#pragma unroll
      for (int k1 = 0; k1 < B; ++k1) xb[(k1 * A + tc) * CW + cw] = v[k1];
      __syncthreads();
      line_stage2<N, +1>(v, tc, [&](int tt, int k1) { return xb[(k1 * A + tt) * CW + cw]; });
#pragma unroll
      for (int j = 0; j < B; ++j) cbuf[cidx(tc + A * j, cl)] = v[j];
    }
  }

  if constexpr (INVERSE) {
    cluster.sync();
    // ---------------- 5. inverse row pass, pulled from the column owners
#pragma unroll 1
    for (int s = 0; s < RPC / RF; ++s) {
      const int a = rank * RPC + s * RF + lr;
      float2 v[B];
#pragma unroll
      for (int j = 0; j < B; ++j) v[j] = rc(j / JPC)[cidx(a, t + A * (j % JPC))];
      line_stage1<N, +1>(v, t, tw);
      __syncwarp();
#pragma unroll
      for (int k1 = 0; k1 < B; ++k1) rs[k1 * (A + 1) + t] = v[k1];
      __syncwarp();
      line_stage2<N, +1>(v, t, [&](int tt, int k1) { return rs[k1 * (A + 1) + tt]; });
#pragma unroll
      for (int j = 0; j < B; ++j) v[j] = cscale(v[j], kInv);
      frame_output_line<N, OP, A, B>(g, r0, r1, psi, a, t, v);
      __syncwarp();
    }
    // the pulled values are consumed before each CTA arrives, so a relaxed
    // barrier suffices to keep the column buffers alive until every pull is done
    cluster_sync_relaxed();
  }

  if (g.err_part) {
    const double sum = block_sum_d(ff_to_double(err), red);
    if (tid == 0) {
      double* ep = g.err_part + (size_t)f * g.err_stride;
      ep[rank] = sum;
      if (rank == 0)
        for (int k = C; k < g.err_stride; ++k) ep[k] = 0.0;   // slots of larger tiles
    }
  }
}

template <int N, int C, int OP>
static int set_cluster_attr() {
  using K = ClusterCfg<N, C>;
  auto fn = cluster_frame_kernel<N, C, OP>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)K::SMEM);
  if (e == cudaSuccess && C > 8) e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) return set_cuda_error(e, "cluster_frame_kernel attributes");
  return PTY_OK;
}

template <int N, int C>
static cudaLaunchConfig_t cluster_config(int nframes, cudaStream_t st, cudaLaunchAttribute* attr) {
  using K = ClusterCfg<N, C>;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nframes * C);
  cfg.blockDim = dim3(K::NT);
  cfg.dynamicSmemBytes = K::SMEM;
  cfg.stream = st;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

template <int N, int C, int OP>
static int launch_cluster(const FrameArgs& a, int nframes, cudaStream_t st) {
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = cluster_config<N, C>(nframes, st, attr);
  cudaError_t e = cudaLaunchKernelEx(&cfg, cluster_frame_kernel<N, C, OP>, a);
  if (e != cudaSuccess) return set_cuda_error(e, "cluster_frame_kernel launch");
  return check_launch("cluster_frame_kernel");
}

// Sets the kernels' attributes and refuses the tile when no cluster of its
// size can be resident on this GPU.
template <int N, int C>
static int prepare_cluster_tile() {
  int rc = PTY_OK;
  if (!rc) rc = set_cluster_attr<N, C, OP_EXIT1>();
  if (!rc) rc = set_cluster_attr<N, C, OP_EXIT7>();
  if (!rc) rc = set_cluster_attr<N, C, OP_PSI1>();
  if (!rc) rc = set_cluster_attr<N, C, OP_PSI7>();
  if (!rc) rc = set_cluster_attr<N, C, OP_DM1>();
  if (!rc) rc = set_cluster_attr<N, C, OP_DM7>();
  if (!rc) rc = set_cluster_attr<N, C, OP_MERR>();
  if (!rc) rc = set_cluster_attr<N, C, OP_INTENS>();
  if (!rc) rc = set_cluster_attr<N, C, OP_MERR_PSI>();
  if (!rc) rc = set_cluster_attr<N, C, OP_BP>();
  if (rc) return rc;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = cluster_config<N, C>(1, nullptr, attr);
  int nclusters = 0;
  cudaError_t e = cudaOccupancyMaxActiveClusters(&nclusters, cluster_frame_kernel<N, C, OP_PSI7>, &cfg);
  if (e != cudaSuccess) return set_cuda_error(e, "cudaOccupancyMaxActiveClusters");
  if (nclusters < 1) return set_error(PTY_ERR_UNSUPPORTED, "no cluster for this frame size fits the GPU");
  return PTY_OK;
}

template <int N, int C>
static int launch_cluster_tile(int op, const FrameArgs& a, int nframes, cudaStream_t st) {
  switch (op) {
    case OP_EXIT1: return launch_cluster<N, C, OP_EXIT1>(a, nframes, st);
    case OP_EXIT7: return launch_cluster<N, C, OP_EXIT7>(a, nframes, st);
    case OP_PSI1: return launch_cluster<N, C, OP_PSI1>(a, nframes, st);
    case OP_PSI7: return launch_cluster<N, C, OP_PSI7>(a, nframes, st);
    case OP_DM1: return launch_cluster<N, C, OP_DM1>(a, nframes, st);
    case OP_DM7: return launch_cluster<N, C, OP_DM7>(a, nframes, st);
    case OP_MERR: return launch_cluster<N, C, OP_MERR>(a, nframes, st);
    case OP_INTENS: return launch_cluster<N, C, OP_INTENS>(a, nframes, st);
    case OP_MERR_PSI: return launch_cluster<N, C, OP_MERR_PSI>(a, nframes, st);
    case OP_BP: return launch_cluster<N, C, OP_BP>(a, nframes, st);
  }
  return set_error(PTY_ERR_ARG, "unknown frame op");
}

}  // namespace pty

// Defines the two entry points of one cluster tile: prepare_cluster_<N>x<C>()
// and launch_cluster_<N>x<C>(op, args, nframes, stream).
#define PTY_CLUSTER_TILE(N, C)                                                              \
  namespace pty {                                                                           \
  int prepare_cluster_##N##x##C() { return prepare_cluster_tile<N, C>(); }                  \
  int launch_cluster_##N##x##C(int op, const FrameArgs& a, int nframes, cudaStream_t st) {  \
    return launch_cluster_tile<N, C>(op, a, nframes, st);                                   \
  }                                                                                         \
  }
