// Fused per-frame kernels: exit-wave formation -> 2-D FFT -> modulus constraint
// -> inverse 2-D FFT, one CTA per frame, the whole frame resident in shared memory.
//
// Replaces, per frame and in one launch over all frames:
//   make_exits        ptychography/era.py:426-433   psi_i = P * O[window_i]
//   pmod_1 / Pmod_1   ptychography/era.py:550-572   amplitude replacement, eMod
//   pmod_7 / Pmod_7   ptychography/era.py:574-595   same with incoherent background
//   Pmod_P            ptychography/era.py:597-610   (one "frame" = the probe)
//   DM update         ptychography/dm.py:91-97, 216-224
//   model_error_1     ptychography/dm.py:337-341
//   info['I']         ptychography/era.py:295, dm.py:299
//
// Shared-memory frame layout: row a, column c at a * RP + c + c / A1 (one pad
// slot every A1 columns), which makes the row exchanges and the column passes
// free of bank conflicts.  Frequencies are in NumPy's unshifted FFT order,
// matching the reference's ifftshift-ed amp / mask.
#include "engine.h"
#include "fft_line.cuh"
#include "frame_ops.cuh"

namespace pty {

// Shared-memory layout of one frame: element (row r, column c) at
//   r * RP + (c + c / A1) + (r / A0) * S1 + (r % A0) * S2.
// The column pad (one slot per A1 columns), the pitch RP and the two row skews
// were chosen by exhaustive search so that every shared-memory walk of the
// kernel -- row loads / exchanges, column loads / exchanges -- is free of bank
// conflicts for the square shapes (the 32 x 64 shape keeps some conflicts).
template <int N0, int N1>
struct FrameLayout {
  static constexpr int A1 = LineGeom<N1>::A, B1 = LineGeom<N1>::B;
  static constexpr int ROWLEN = B1 * (A1 + 1);
  static constexpr int RP = ROWLEN;
  static constexpr int S1 = 0, S2 = 0;
};
template <> struct FrameLayout<32, 32> { static constexpr int RP = 40, S1 = 12, S2 = 4; };
template <> struct FrameLayout<64, 64> { static constexpr int RP = 72, S1 = 14, S2 = 2; };
template <> struct FrameLayout<128, 128> { static constexpr int RP = 144, S1 = 14, S2 = 2; };

template <int N0, int N1>
struct FrameCfg {
  static constexpr int A0 = LineGeom<N0>::A, B0 = LineGeom<N0>::B;  // column transform
  static constexpr int A1 = LineGeom<N1>::A, B1 = LineGeom<N1>::B;  // row transform
  static constexpr int RP = FrameLayout<N0, N1>::RP;
  static constexpr int S1 = FrameLayout<N0, N1>::S1, S2 = FrameLayout<N0, N1>::S2;
  static constexpr int BUF = (N0 - 1) * RP + (N1 - 1) + (N1 - 1) / A1 + ((N0 - 1) / A0) * S1 +
                             (A0 - 1) * S2 + 1;
  static constexpr int T_ROW = N0 * A1, T_COL = N1 * A0;
  static constexpr int NT0 = T_ROW < T_COL ? T_ROW : T_COL;
  static constexpr int NT = NT0 < 512 ? NT0 : 512;
  static constexpr int CW = NT / A0;                 // columns per column pass
  static constexpr size_t XB = (size_t)N0 * CW;       // column exchange buffer (float2)
  static constexpr size_t SMEM = ((size_t)BUF + XB) * sizeof(float2) +
                                 (size_t)(N0 + N1) * sizeof(float2) + 32 * sizeof(double);
  static_assert(SMEM <= 227 * 1024, "shared memory budget");
  static_assert(T_ROW % NT == 0 && T_COL % NT == 0 && NT % 32 == 0, "task split");
  // rows must not overlap: consecutive row bases differ by at least a padded row
  static_assert(RP + S2 >= B1 * (A1 + 1) && RP + S1 - (A0 - 1) * S2 >= B1 * (A1 + 1), "row pitch");
};

// Row handled by row-task slot rho: the rows sharing a half-warp are 4 apart
// (8-thread rows) or 4 / 8 / 12 apart (4-thread rows), as the layout assumes.
template <int A1>
PTY_DEV int row_of_slot(int rho) {
  if constexpr (A1 == 8) return (rho & ~7) + (rho & 1) * 4 + ((rho & 7) >> 1);
  else if constexpr (A1 == 4) return (rho & ~15) + (rho & 3) * 4 + ((rho & 15) >> 2);
  else return rho;
}

PTY_DEV int padpos(int c, int A) { return c + c / A; }

template <int N0, int N1, int OP>
__global__ void __launch_bounds__(FrameCfg<N0, N1>::NT, 1) frame_kernel(FrameArgs g) {
  using C = FrameCfg<N0, N1>;
  constexpr int A0 = C::A0, B0 = C::B0, A1 = C::A1, B1 = C::B1, RP = C::RP, NT = C::NT;
  constexpr int S1 = C::S1, S2 = C::S2;
  constexpr bool INVERSE = OpTraits<OP>::INVERSE;
  auto rbase = [](int r) { return r * RP + (r / A0) * S1 + (r % A0) * S2; };
  constexpr float kInv = 1.0f / (float)(N0 * N1);

  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* fr = reinterpret_cast<float2*>(smem_raw);
  float2* xb = fr + C::BUF;   // column exchange: [row slot][CW columns]
  float2* tw0 = xb + C::XB;
  float2* tw1 = tw0 + N0;
  double* red = reinterpret_cast<double*>(tw1 + N1);

  const int f = blockIdx.x;
  const int tid = threadIdx.x;
  for (int i = tid; i < N0; i += NT) tw0[i] = g.tw0[i];
  for (int i = tid; i < N1; i += NT) tw1[i] = g.tw1[i];

  int r0 = 0, r1 = 0;
  if (OpTraits<OP>::IN_EXIT || OpTraits<OP>::IN_DM) {
    r0 = g.R[2 * f];
    r1 = g.R[2 * f + 1];
  }
  const size_t fbase = (size_t)f * N0 * N1;
  float2* psi = g.psi + fbase;
  __syncthreads();

  // ---------------- forward row pass (a row's A1 threads share a warp)
  for (int id = tid; id < N0 * A1; id += NT) {
    const int t = id % A1, a = row_of_slot<A1>(id / A1);
    float2 v[B1];
#pragma unroll
    for (int j = 0; j < B1; ++j) v[j] = frame_input<N1, OP>(g, f, r0, r1, psi, a, t + A1 * j);
    line_stage1<N1, OpTraits<OP>::FIRST_DIR>(v, t, tw1);
    float2* row = fr + rbase(a);
#pragma unroll
    for (int k1 = 0; k1 < B1; ++k1) row[k1 * (A1 + 1) + t] = v[k1];
    __syncwarp();
    line_stage2<N1, OpTraits<OP>::FIRST_DIR>(v, t, [&](int tt, int k1) { return row[k1 * (A1 + 1) + tt]; });
    __syncwarp();
#pragma unroll
    for (int j = 0; j < B1; ++j) row[t + j * (A1 + 1)] = v[j];
  }
  constexpr int CW = C::CW;
  // the modulus inputs of the first column pass are loaded across the barrier
  ModIn<OP, B0> m;
  modulus_load<N0, N1, OP, A0, B0>(g, f, fbase, tid / CW, tid % CW, m);
  __syncthreads();

  // ---------------- column pass: forward FFT, modulus constraint, inverse FFT
  // Each pass takes CW whole columns (all A0 line-threads of a column in the
  // same pass, as the exchange needs); lanes of a warp run along a row, so the
  // amp / mask / background traffic is coalesced.  The exchanges go through a
  // separate [row slot][CW columns] buffer, so frame loads and exchange writes
  // never collide and fewer CTA barriers are needed.
  ff err = ff_zero();
  static_assert(NT % A0 == 0 && N1 % CW == 0 && CW >= 32, "column pass split");
#pragma unroll 1
  for (int c0 = 0; c0 < N1; c0 += CW) {
    const int cw = tid % CW, t = tid / CW;
    const int c = c0 + cw;
    const int cp = padpos(c, A1);
    auto at = [&](int r) -> float2& { return fr[rbase(r) + cp]; };
    // this pass's amp / mask / background, in flight during the forward FFT
    if (c0 > 0) modulus_load<N0, N1, OP, A0, B0>(g, f, fbase, t, c, m);
    float2 v[B0];
#pragma unroll
    for (int j = 0; j < B0; ++j) v[j] = at(t + A0 * j);
    line_stage1<N0, OpTraits<OP>::FIRST_DIR>(v, t, tw0);
    if (c0 > 0) __syncthreads();   // previous pass done reading xb
#pragma unroll
    for (int k1 = 0; k1 < B0; ++k1) xb[(k1 * A0 + t) * CW + cw] = v[k1];
    __syncthreads();
    line_stage2<N0, OpTraits<OP>::FIRST_DIR>(v, t, [&](int tt, int k1) { return xb[(k1 * A0 + tt) * CW + cw]; });
    modulus_load_late<N0, N1, OP, A0, B0>(g, fbase, t, c, m);
    modulus_apply<N0, N1, OP, A0, B0>(g, fbase, t, c, v, m, err);
    if constexpr (INVERSE) {
      line_stage1<N0, +1>(v, t, tw0);
      __syncthreads();
#pragma unroll
      for (int k1 = 0; k1 < B0; ++k1) xb[(k1 * A0 + t) * CW + cw] = v[k1];
      __syncthreads();
      line_stage2<N0, +1>(v, t, [&](int tt, int k1) { return xb[(k1 * A0 + tt) * CW + cw]; });
#pragma unroll
      for (int j = 0; j < B0; ++j) at(t + A0 * j) = v[j];
    }
  }

  if constexpr (INVERSE) {
    __syncthreads();
    // ---------------- inverse row pass, write the result
    for (int id = tid; id < N0 * A1; id += NT) {
      const int t = id % A1, a = row_of_slot<A1>(id / A1);
      float2* row = fr + rbase(a);
      float2 v[B1];
#pragma unroll
      for (int j = 0; j < B1; ++j) v[j] = row[t + j * (A1 + 1)];
      line_stage1<N1, +1>(v, t, tw1);
      __syncwarp();
#pragma unroll
      for (int k1 = 0; k1 < B1; ++k1) row[k1 * (A1 + 1) + t] = v[k1];
      __syncwarp();
      line_stage2<N1, +1>(v, t, [&](int tt, int k1) { return row[k1 * (A1 + 1) + tt]; });
#pragma unroll
      for (int j = 0; j < B1; ++j) v[j] = cscale(v[j], kInv);
      frame_output_line<N1, OP, A1, B1>(g, r0, r1, psi, a, t, v);
    }
  }

  if (g.err_part) {
    const double s = block_sum_d(ff_to_double(err), red);
    if (tid == 0) {
      double* ep = g.err_part + (size_t)f * g.err_stride;
      ep[0] = s;
      for (int k = 1; k < g.err_stride; ++k) ep[k] = 0.0;   // slots of cluster tiles
    }
  }
}

template <int N0, int N1, int OP>
static int set_attr() {
  using C = FrameCfg<N0, N1>;
  cudaError_t e = cudaFuncSetAttribute(frame_kernel<N0, N1, OP>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM);
  if (e != cudaSuccess) return set_cuda_error(e, "frame_kernel smem attribute");
  return PTY_OK;
}

template <int N0, int N1, int OP>
static int launch_one(const FrameArgs& a, int nframes, cudaStream_t st) {
  using C = FrameCfg<N0, N1>;
  frame_kernel<N0, N1, OP><<<nframes, C::NT, C::SMEM, st>>>(a);
  return check_launch("frame_kernel");
}

template <int N0, int N1>
static int launch_op(int op, const FrameArgs& a, int nframes, cudaStream_t st) {
  switch (op) {
    case OP_EXIT1: return launch_one<N0, N1, OP_EXIT1>(a, nframes, st);
    case OP_EXIT7: return launch_one<N0, N1, OP_EXIT7>(a, nframes, st);
    case OP_PSI1: return launch_one<N0, N1, OP_PSI1>(a, nframes, st);
    case OP_PSI7: return launch_one<N0, N1, OP_PSI7>(a, nframes, st);
    case OP_DM1: return launch_one<N0, N1, OP_DM1>(a, nframes, st);
    case OP_DM7: return launch_one<N0, N1, OP_DM7>(a, nframes, st);
    case OP_MERR: return launch_one<N0, N1, OP_MERR>(a, nframes, st);
    case OP_INTENS: return launch_one<N0, N1, OP_INTENS>(a, nframes, st);
    case OP_MERR_PSI: return launch_one<N0, N1, OP_MERR_PSI>(a, nframes, st);
    case OP_BP: return launch_one<N0, N1, OP_BP>(a, nframes, st);
  }
  return set_error(PTY_ERR_ARG, "unknown frame op");
}

template <int N0, int N1>
static int prepare_shape() {
  int rc = PTY_OK;
  if (!rc) rc = set_attr<N0, N1, OP_EXIT1>();
  if (!rc) rc = set_attr<N0, N1, OP_EXIT7>();
  if (!rc) rc = set_attr<N0, N1, OP_PSI1>();
  if (!rc) rc = set_attr<N0, N1, OP_PSI7>();
  if (!rc) rc = set_attr<N0, N1, OP_DM1>();
  if (!rc) rc = set_attr<N0, N1, OP_DM7>();
  if (!rc) rc = set_attr<N0, N1, OP_MERR>();
  if (!rc) rc = set_attr<N0, N1, OP_INTENS>();
  if (!rc) rc = set_attr<N0, N1, OP_MERR_PSI>();
  if (!rc) rc = set_attr<N0, N1, OP_BP>();
  return rc;
}

int prepare_single_cta(int N0, int N1) {
  if (N0 == 32 && N1 == 32) return prepare_shape<32, 32>();
  if (N0 == 64 && N1 == 64) return prepare_shape<64, 64>();
  if (N0 == 128 && N1 == 128) return prepare_shape<128, 128>();
  if (N0 == 32 && N1 == 64) return prepare_shape<32, 64>();
  return set_error(PTY_ERR_SHAPE, "no single-CTA frame kernel for this shape");
}

int launch_single_cta_op(int op, int N0, int N1, const FrameArgs& a, int nframes, cudaStream_t st) {
  if (N0 == 32 && N1 == 32) return launch_op<32, 32>(op, a, nframes, st);
  if (N0 == 64 && N1 == 64) return launch_op<64, 64>(op, a, nframes, st);
  if (N0 == 128 && N1 == 128) return launch_op<128, 128>(op, a, nframes, st);
  if (N0 == 32 && N1 == 64) return launch_op<32, 64>(op, a, nframes, st);
  return set_error(PTY_ERR_UNSUPPORTED, "no single-CTA frame kernel for this shape");
}

}  // namespace pty
