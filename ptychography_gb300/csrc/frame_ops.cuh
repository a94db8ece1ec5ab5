// Per-pixel pieces of the fused frame kernels, shared by the one-CTA-per-frame
// kernel (frame_kernels.cu) and the cluster-per-frame kernel (cluster_kernels.cu):
//   frame_input   -- the wave entering the forward FFT at detector pixel (a, b)
//   frame_modulus -- the constraint applied to F at frequency (kr, kc)
//   frame_output  -- what is written back after the inverse FFT
#pragma once
#include "engine.h"

namespace pty {

template <int OP>
struct OpTraits {
  static constexpr bool IN_EXIT = (OP == OP_EXIT1 || OP == OP_EXIT7 || OP == OP_MERR || OP == OP_INTENS);
  static constexpr bool IN_DM = (OP == OP_DM1 || OP == OP_DM7);
  static constexpr bool INVERSE = !(OP == OP_MERR || OP == OP_MERR_PSI || OP == OP_INTENS);
};

// exit wave P * O[window] (era.py:426-433) at frame pixel (a, b)
template <int N1>
PTY_DEV float2 exit_wave(const FrameArgs& g, int r0, int r1, int a, int b) {
  int u = a - r0, v = b - r1;
  if (u >= g.U) u -= g.U;
  if (v >= g.V) v -= g.V;
  return cmul(__ldg(&g.O[(size_t)u * g.V + v]), __ldg(&g.P[a * N1 + b]));
}

template <int N1, int OP>
PTY_DEV float2 frame_input(const FrameArgs& g, int r0, int r1, const float2* psi, int a, int b) {
  if constexpr (OpTraits<OP>::IN_EXIT) {
    return exit_wave<N1>(g, r0, r1, a, b);
  } else if constexpr (OpTraits<OP>::IN_DM) {
    // dm.py:94-95: e1 = psi - ex0 ; x = ex0 - e1  (= 2 ex0 - psi, rounded as the reference)
    const float2 ex0 = exit_wave<N1>(g, r0, r1, a, b);
    const float2 e1 = csub(psi[a * N1 + b], ex0);
    return csub(ex0, e1);
  } else {
    return psi[a * N1 + b];
  }
}

// r is the inverse transform already scaled by 1 / (N0 N1)
template <int N1, int OP>
PTY_DEV void frame_output(const FrameArgs& g, int r0, int r1, float2* psi, int a, int b, float2 r) {
  if constexpr (OpTraits<OP>::IN_DM) {
    // dm.py:94-97: psi_new = (psi - ex0) + Pmod(2 ex0 - psi)
    const float2 ex0 = exit_wave<N1>(g, r0, r1, a, b);
    const float2 e1 = csub(psi[a * N1 + b], ex0);
    psi[a * N1 + b] = cadd(e1, r);
  } else {
    psi[a * N1 + b] = r;
  }
}

template <int N0, int N1, int OP>
PTY_DEV void frame_modulus(const FrameArgs& g, int f, size_t fbase, int kr, int kc, float2& F, ff& err) {
  const int pix = kr * N1 + kc;
  const float msk = g.mask ? (float)g.mask[pix] : 1.0f;
  if constexpr (OP == OP_INTENS) {
    const int sr = (kr + N0 / 2) % N0, sc = (kc + N1 / 2) % N1;   // fftshift, era.py:295
    g.out_real[fbase + (size_t)sr * N1 + sc] = cabs2(F);
  } else {
    const float am = g.amp[(size_t)g.amp_stride * f + pix];
    if constexpr (OP == OP_EXIT1 || OP == OP_PSI1 || OP == OP_DM1) {
      // era.py:561-571: |F| + alpha, masked pixels keep F
      const float mag = sqrtf(cabs2(F)) + g.alpha;
      if (g.err_part) {
        const float d = mag - am;
        err = ff_add(err, d * d * msk);
      }
      const float fac = (msk != 0.f) ? am / mag : 1.0f;
      F = cscale(F, fac);
    } else if constexpr (OP == OP_EXIT7 || OP == OP_PSI7) {
      // era.py:584-594: sqrt(|F|^2 + b^2 + alpha), masked pixels zeroed
      const float b = g.bg_in[(size_t)g.bg_stride * f + pix];
      const float mag = sqrtf(cabs2(F) + b * b + g.alpha);
      if (g.err_part) {
        const float d = mag - am;
        err = ff_add(err, d * d * msk);
      }
      const float fac = msk * am / mag;
      F = cscale(F, fac);
      g.bg_out[fbase + pix] = b * fac;
    } else if constexpr (OP == OP_DM7) {
      // dm.py:219-224 on the background: g1 = g - b0 ; tb = b0 - g1 ; g = g1 + Pmod7(tb)
      const float gs = g.bg_out[fbase + pix];
      const float b0 = g.b0[pix];
      const float g1 = gs - b0;
      const float tb = b0 - g1;
      const float mag = sqrtf(cabs2(F) + tb * tb + g.alpha);
      const float fac = msk * am / mag;
      F = cscale(F, fac);
      g.bg_out[fbase + pix] = g1 + tb * fac;
    } else if constexpr (OP == OP_MERR || OP == OP_MERR_PSI) {
      // dm.py:338-340, no alpha
      const float b = g.bg_in ? g.bg_in[(size_t)g.bg_stride * f + pix] : 0.0f;
      const float mag = sqrtf(cabs2(F) + b * b);
      const float d = mag - am;
      err = ff_add(err, msk * (d * d));
    }
  }
}

}  // namespace pty
